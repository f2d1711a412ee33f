"""CPU: the even/odd decomposition used by the two-pass reduced product.

The subgroup H of the layer group that preserves even/odd sites acts on the
even half e and odd half o as two dihedral actions.  Check that every H element
maps each state into its own orbit under the reference group, and that H has
L (2L with spin flip) distinct elements."""
import random

import pytest


def rotr(s, n, d):
    d %= n
    return ((s >> d) | ((s & ((1 << d) - 1)) << (n - d))) if d else s


def brev(s, n):
    return int(format(s, "0%db" % n)[::-1], 2)


def split(s, L):
    e = o = 0
    for a in range(L // 2):
        e |= ((s >> (2 * a)) & 1) << a
        o |= ((s >> (2 * a + 1)) & 1) << a
    return e, o


def join(e, o, m):
    s = 0
    for a in range(m):
        s |= ((e >> a) & 1) << (2 * a)
        s |= ((o >> a) & 1) << (2 * a + 1)
    return s


def orbit(s, L, flip):
    mask = (1 << L) - 1
    out = set()
    for k in range(L):
        a = rotr(s, L, k)
        b = brev(a, L)
        out |= {a, b}
        if flip:
            out |= {~a & mask, ~b & mask}
    return out


def act(g, e, o, m):
    """Same element numbering as act_e / act_o in latttmat_gb300/csrc/tm_eo.cu."""
    j, refl, fl = g % m, (g // m) % 2, g // (2 * m)
    mk = (1 << m) - 1
    if refl:
        e2 = rotr(brev(rotr(e, m, j), m), m, m - 1)
        o2 = brev(rotr(o, m, j), m)
    else:
        e2, o2 = rotr(e, m, j), rotr(o, m, j)
    if fl:
        e2 ^= mk
        o2 ^= mk
    return e2, o2


@pytest.mark.parametrize("L", [8, 12, 16, 20])
@pytest.mark.parametrize("flip", [0, 1])
def test_even_odd_subgroup(L, flip):
    m = L // 2
    ng = 2 * m * (2 if flip else 1)
    rng = random.Random(L * 10 + flip)
    maps = set()
    for g in range(ng):
        probe = tuple(join(*act(g, *split(s, L), m), m) for s in (rng.getrandbits(L) for _ in range(40)))
        for _ in range(30):
            s = rng.getrandbits(L)
            s2 = join(*act(g, *split(s, L), m), m)
            assert s2 in orbit(s, L, flip)
        maps.add(tuple(join(*act(g, *split(s, L), m), m) for s in range(0, 1 << L, max(1, (1 << L) // 4096))))
    assert len(maps) == ng


# ---- run-start forms of the periodic X-2D group (L <= 32), as the GPU
# orbit-table and map kernels compute them: the smallest image starts with a
# longest run of zeros (or, with the flip, of ones), so only the rotations that
# bring such a run to the front are compared.

def _rotr_m(x, L, k, mask):
    return ((x >> k) | (x << (L - k))) & mask if k else x


def _run_starts(y, L, k, mask):
    """bits where a cyclic run of >= k ones of y starts (every bit for k=0)"""
    t = mask
    for q in range(k):
        t &= _rotr_m(y, L, q, mask)
    return t


def _longest_run(y, L, mask):
    t, k = y, 1
    while True:
        nt = t & _rotr_m(y, L, k, mask)
        if not nt:
            return k, t
        t, k = nt, k + 1


def _images(s, L, flip):
    mask = (1 << L) - 1
    out = []
    for k in range(L):
        a = _rotr_m(s, L, k, mask)
        b = brev(a, L)
        out += [a, b] + ([a ^ mask, b ^ mask] if flip else [])
    return out


def _canon_runs(s, L, flip):
    mask = (1 << L) - 1
    if s == 0 or (flip and s == mask):
        return 0
    if s == mask:
        return s
    r = brev(s, L)
    Z, zs = _longest_run(~s & mask, L, mask)
    O, os_ = _longest_run(s, L, mask) if flip else (-1, 0)
    best = mask
    cands = []
    if Z >= O:
        cands += [(s, zs, Z, False), (r, _longest_run(~r & mask, L, mask)[1], Z, False)]
    if flip and O >= Z:
        cands += [(s, os_, O, True), (r, _longest_run(r, L, mask)[1], O, True)]
    for v, t, k0, inv in cands:
        for i in range(L):
            if (t >> i) & 1:
                a = _rotr_m(v, L, (i + k0) % L, mask)
                best = min(best, (a ^ mask) if inv else a)
    return best


def _rep_runs(s, L, flip):
    """(is the orbit minimum, number of group elements fixing s)"""
    mask = (1 << L) - 1
    if s == 0:
        return True, 2 * L
    z = L - s.bit_length()
    r = brev(s, L)
    f = 0
    for v, inv in [(s, False), (r, False)] + ([(s, True), (r, True)] if flip else []):
        t = _run_starts(v if inv else (~v & mask), L, z, mask)
        for i in range(L):
            if (t >> i) & 1:
                a = _rotr_m(v, L, (i + z) % L, mask)
                if inv:
                    a ^= mask
                if a < s:
                    return False, 0
                f += a == s
    return True, f


@pytest.mark.parametrize("flip", [0, 1])
def test_run_start_forms_exhaustive(flip):
    for L in range(2, 13):
        for s in range(1 << L):
            ims = _images(s, L, flip)
            assert _canon_runs(s, L, flip) == min(ims)
            rep, fix = _rep_runs(s, L, flip)
            assert rep == (min(ims) == s)
            if rep:
                assert fix == sum(im == s for im in ims)


@pytest.mark.parametrize("flip", [0, 1])
def test_run_start_forms_sampled_l32(flip):
    rng = random.Random(7 + flip)
    L = 32
    for _ in range(3000):
        s = rng.getrandbits(L) >> rng.randrange(L)
        ims = _images(s, L, flip)
        assert _canon_runs(s, L, flip) == min(ims)
        rep, fix = _rep_runs(s, L, flip)
        assert rep == (min(ims) == s)
        if rep:
            assert fix == sum(im == s for im in ims)


def _word_rejected(w, L, flip):
    """The orbit-table kernel's screen of the 32 states w*32 + b: a run of
    more than z zeros (with the flip: or ones) inside their shared bits
    [5, L), z their common leading-zero count, rules the word out."""
    if w == 0 or L <= 6:
        return False
    up = w << 5
    z = L - up.bit_length()
    if z + 1 > L - 5:
        return False
    umask = ((1 << L) - 1) & ~31

    def run(y, k):
        t, ln = y, 1
        while 2 * ln <= k:
            t &= t >> ln
            ln *= 2
        if k > ln:
            t &= t >> (k - ln)
        return t != 0

    return run(~up & umask, z + 1) or bool(flip and run(up & umask, z + 1))


@pytest.mark.parametrize("flip", [0, 1])
def test_word_screen_never_drops_a_representative(flip):
    np = pytest.importorskip("numpy")
    for L in range(7, 17):
        mask = (1 << L) - 1
        s = np.arange(1 << L, dtype=np.int64)
        rev = np.zeros_like(s)
        for i in range(L):
            rev |= ((s >> i) & 1) << (L - 1 - i)
        best = s.copy()
        for k in range(L):
            a = ((s >> k) | (s << (L - k))) & mask
            b = ((rev >> k) | (rev << (L - k))) & mask
            for im in [a, b] + ([a ^ mask, b ^ mask] if flip else []):
                best = np.minimum(best, im)
        words = set((np.nonzero(best == s)[0] >> 5).tolist())
        assert not [w for w in words if _word_rejected(w, L, flip)]
        # and the screen does real work (over 60% of the words from L = 12 on)
        if L >= 12:
            nw = (1 << L) >> 5
            assert sum(_word_rejected(w, L, flip) for w in range(nw)) > 0.6 * nw
