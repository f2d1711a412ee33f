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
