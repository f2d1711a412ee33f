/*
 * tm_oracle.c -- CPU restatement of LattTMat's transfer-matrix hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the oracle: the tests, smoke() and
 * bench.py's CPU-baseline leg call it to check the GPU results or as the
 * timed CPU reference.  The GPU product path never calls it.
 *
 * Each function restates the reference algorithm it cites (LattTMat TMat/ sources)
 * in plain C99 + OpenMP, with the same loop structure and arithmetic order:
 *   - serial bitset orbit scans (orbit minima, orbit sizes),
 *   - genTvec Boltzmann weights,
 *   - perform_op of the full operators (XAT, XDT, ZBT and its transpose),
 *   - perform_op of the reduced operators with the reference's leading-bit
 *     slicing (XAM, XDM, ZBM and its transpose, 3D XAM),
 *   - moments / phys_extend.
 * It is pinned against the golden fixtures in tests/golden (outputs of the
 * reference compiled from its own sources).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

typedef uint64_t st_t;

/* ------------------------------------------------------------ bit helpers */
/* TMat/utility.hpp:65-84 */
static inline double powdi(const double* a, int b) {
  double r = 1.0, t;
  if (b < 0) {
    b = -b;
    t = a[0];
  } else {
    t = a[1];
  }
  while (b) {
    if (b & 1) r *= t;
    t *= t;
    b >>= 1;
  }
  return r;
}
static inline int popc(st_t s) { return __builtin_popcountll(s); }
static inline int nanti2(st_t a, st_t b) { return __builtin_popcountll(a ^ b); }
/* TMat/utility.hpp:104-115 */
static inline int bzexp1(st_t s, int n) { return 2 * popc(s) - n; }
static inline int bzexp2(st_t a, st_t b, int n) { return 2 * popc(a ^ b) - n; }
/* TMat/utility.hpp:120-131 */
static inline st_t rotr(st_t s, int n, int d) { return d ? (s >> d | (s & ((1ull << d) - 1)) << (n - d)) : s; }
static inline st_t rotl(st_t s, int n, int d) { return d ? (((s << d) & ((1ull << n) - 1)) | (s >> (n - d))) : s; }
/* TMat/utility.hpp:154-157 */
static inline double bzexpn(int nspin, int nanti, double J) { return J * (2.0 * nanti - nspin); }
/* TMat/utility.cpp:17-31 */
static st_t brev(st_t s, int nbit) {
  s = ((s >> 1) & 0x5555555555555555ull) | ((s & 0x5555555555555555ull) << 1);
  s = ((s >> 2) & 0x3333333333333333ull) | ((s & 0x3333333333333333ull) << 2);
  s = ((s >> 4) & 0x0f0f0f0f0f0f0f0full) | ((s & 0x0f0f0f0f0f0f0f0full) << 4);
  s = ((s >> 8) & 0x00ff00ff00ff00ffull) | ((s & 0x00ff00ff00ff00ffull) << 8);
  s = ((s >> 16) & 0x0000ffff0000ffffull) | ((s & 0x0000ffff0000ffffull) << 16);
  s = (s >> 32) | (s << 32);
  return s >> (64 - nbit);
}
/* TMat/utility.cpp:35-47 */
static int nnode(st_t s, int n, int bc) {
  st_t t = s >> 1;
  if (!bc)
    t |= (s & 1) << (n - 1);
  else
    t |= (s & (st_t)(n - 1)) << 1;
  return popc(s ^ t);
}
/* TMat/utility.cpp:52-120 */
static st_t rff3(st_t s, int s1, int s2, int d) {
  st_t mask = (1ull << s2) - 1, r = 0;
  for (int i = 0; i < s1; ++i) {
    r |= rotr(s & mask, s2, d) << (i * s2);
    s >>= s2;
  }
  return r;
}
static st_t dff3(st_t s, int s1, int s2, int d) {
  st_t mask = (1ull << (s2 * d)) - 1;
  return (s >> (s2 * d)) | ((s & mask) << ((s1 - d) * s2));
}
static st_t rot3(st_t s, int size) {
  st_t r = 0;
  for (int a = 0; a < size; ++a)
    for (int b = 0; b < size; ++b)
      if (s & (1ull << (a * size + b))) r |= 1ull << ((b + 1) * size - (a + 1));
  return r;
}
static st_t refl3(st_t s, int s1, int s2, int ax) {
  st_t mask = (1ull << s2) - 1, r = 0;
  if (!ax) {
    for (int i = 0; i < s1; ++i) {
      r |= brev(s & mask, s2) << (i * s2);
      s >>= s2;
    }
  } else {
    for (int i = 0; i < s1; ++i) {
      r <<= s2;
      r |= s & mask;
      s >>= s2;
    }
  }
  return r;
}

/* ------------------------------------------------------------ bitset */
/* TMat/tmat.hpp:573-607 */
typedef struct {
  uint64_t* w;
} bits_t;
static bits_t bits_new(int size) {
  bits_t b;
  size_t nchunk = size <= 6 ? 1 : (1ull << (size - 6));
  b.w = (uint64_t*)calloc(nchunk, 8);
  return b;
}
static inline int bget(bits_t b, st_t s) { return (b.w[s >> 6] >> (s & 63)) & 1; }
static inline void bset(bits_t b, st_t s) { b.w[s >> 6] |= 1ull << (s & 63); }

/* growable orbit table */
typedef struct {
  st_t* idx;
  uint16_t* dup;
  int64_t n, cap;
} table_t;
static void tpush(table_t* t, st_t s) {
  if (t->n == t->cap) {
    t->cap = t->cap ? 2 * t->cap : 1024;
    t->idx = (st_t*)realloc(t->idx, t->cap * sizeof(st_t));
    t->dup = (uint16_t*)realloc(t->dup, t->cap * sizeof(uint16_t));
  }
  t->idx[t->n] = s;
  t->dup[t->n] = 0;
  t->n++;
}

/* genX2DDuplist, TMat/tmatreduce.cpp:19-111 */
static void gen_x2d(int size, int bc, int cen, table_t* t) {
  st_t nstate = 1ull << size, mask = nstate - 1, ns, nm;
  bits_t buf = bits_new(size);
  for (st_t s = 0; s < nstate; ++s) {
    if (bget(buf, s)) continue;
    tpush(t, s);
    uint16_t* d = &t->dup[t->n - 1];
    if (!bc) {
      for (ns = s; !bget(buf, ns); ns = ns >> 1 | (ns & 1) << (size - 1)) {
        ++*d;
        bset(buf, ns);
        if (cen) {
          nm = ~ns & mask;
          if (!bget(buf, nm)) {
            ++*d;
            bset(buf, nm);
          }
        }
      }
      for (ns = brev(s, size); !bget(buf, ns); ns = ns >> 1 | (ns & 1) << (size - 1)) {
        ++*d;
        bset(buf, ns);
        if (cen) {
          nm = ~ns & mask;
          if (!bget(buf, nm)) {
            ++*d;
            bset(buf, nm);
          }
        }
      }
    } else {
      bset(buf, s);
      ++*d;
      ns = brev(s, size);
      if (ns != s) {
        ++*d;
        bset(buf, ns);
      }
      if (cen) {
        nm = ~s & mask;
        if (!bget(buf, nm)) {
          ++*d;
          bset(buf, nm);
        }
        nm = ~ns & mask;
        if (!bget(buf, nm)) {
          ++*d;
          bset(buf, nm);
        }
      }
    }
  }
  free(buf.w);
}

/* genZ2DDuplist, TMat/tmatreduce.cpp:242-334 (periodic form, as ZBM uses) */
static void gen_z2d(int size, int cen, table_t* t) {
  st_t nstate = 1ull << size, mask = nstate - 1, ns, nm;
  bits_t buf = bits_new(size);
  for (st_t s = 0; s < nstate; ++s) {
    if (bget(buf, s)) continue;
    tpush(t, s);
    uint16_t* d = &t->dup[t->n - 1];
    for (ns = s; !bget(buf, ns); ns = ns >> 2 | (ns & 3) << (size - 2)) {
      ++*d;
      bset(buf, ns);
      if (cen) {
        nm = ~ns & mask;
        if (!bget(buf, nm)) {
          ++*d;
          bset(buf, nm);
        }
      }
    }
    for (ns = brev(s >> 1 | (s & 1) << (size - 1), size); !bget(buf, ns); ns = ns >> 2 | (ns & 3) << (size - 2)) {
      ++*d;
      bset(buf, ns);
      if (cen) {
        nm = ~ns & mask;
        if (!bget(buf, nm)) {
          ++*d;
          bset(buf, nm);
        }
      }
    }
  }
  free(buf.w);
}

/* genX3DDuplist, TMat/tmat3d.cpp:17-98 */
static void gen_x3d(int s1, int s2, int cen, int rotf, table_t* t) {
  int size = s1 * s2;
  st_t nstate = 1ull << size, mask = nstate - 1;
  bits_t buf = bits_new(size);
  for (st_t s = 0; s < nstate; ++s) {
    if (bget(buf, s)) continue;
    tpush(t, s);
    uint16_t* d = &t->dup[t->n - 1];
    st_t rs = s;
    int rst = 0;
    do {
      st_t cs = rs;
      int cst = 0;
      do {
        st_t m1 = cs;
        int m1s = 0;
        do {
          st_t m2 = m1;
          int m2s = 0;
          do {
            for (st_t o1 = m2; !bget(buf, o1); o1 = rff3(o1, s1, s2, 1))
              for (st_t o2 = o1; !bget(buf, o2); o2 = dff3(o2, s1, s2, 1)) {
                bset(buf, o2);
                ++*d;
              }
            if (!m2s) {
              m2s = 1;
              m2 = refl3(m2, s1, s2, 1);
            } else
              break;
          } while (!bget(buf, m2));
          if (!m1s) {
            m1s = 1;
            m1 = refl3(m1, s1, s2, 0);
          } else
            break;
        } while (!bget(buf, m1));
        if (!cst && cen) {
          cst = 1;
          cs = ~cs & mask;
        } else
          break;
      } while (!bget(buf, cs));
      if (!rst && rotf) {
        rst = 1;
        rs = rot3(rs, s1);
      } else
        break;
    } while (!bget(buf, rs));
  }
  free(buf.w);
}

/* genY2DDuplist, TMat/tmatreduce.cpp:113-240: orbits of two-layer states
 * (left layer in the high L bits) under simultaneous translation, reflection
 * and (cen) spin flip of both layers; dup = orbit size; swp[r] = index of the
 * orbit holding the layer-swapped states of orbit r. */
static st_t y_act(st_t s, int L, int t, int refl, int flip) {
  st_t mask = (1ull << L) - 1, l = s >> L, r = s & mask;
  if (refl) {
    l = brev(l, L);
    r = brev(r, L);
  }
  if (flip) {
    l = ~l & mask;
    r = ~r & mask;
  }
  return rotr(l, L, t) << L | rotr(r, L, t);
}
static st_t y_swap(st_t s, int L) { return (s & ((1ull << L) - 1)) << L | s >> L; }

static int64_t lower_bound_u64(const st_t* a, int64_t n, st_t v) {
  int64_t lo = 0, hi = n;
  while (lo < hi) {
    int64_t mid = (lo + hi) / 2;
    if (a[mid] < v) lo = mid + 1; else hi = mid;
  }
  return lo;
}

static void gen_y2d(int L, int cen, table_t* t, int64_t** swp_out) {
  st_t nstate = 1ull << (2 * L);
  bits_t buf = bits_new(2 * L);
  st_t* mins = NULL;
  int64_t cap = 0;
  for (st_t s = 0; s < nstate; ++s) {
    if (bget(buf, s)) continue;
    tpush(t, s);
    if (t->n > cap) {
      cap = t->cap;
      mins = (st_t*)realloc(mins, cap * sizeof(st_t));
    }
    st_t m = y_swap(s, L);
    uint16_t d = 0;
    for (int f = 0; f <= cen; ++f)
      for (int rf = 0; rf < 2; ++rf)
        for (int sh = 0; sh < L; ++sh) {
          st_t g = y_act(s, L, sh, rf, f);
          if (!bget(buf, g)) {
            bset(buf, g);
            ++d;
          }
          st_t w = y_swap(g, L);
          if (w < m) m = w;
        }
    t->dup[t->n - 1] = d;
    mins[t->n - 1] = m;
  }
  int64_t* swp = (int64_t*)malloc(t->n * sizeof(int64_t));
  for (int64_t r = 0; r < t->n; ++r) swp[r] = lower_bound_u64(t->idx, t->n, mins[r]);
  *swp_out = swp;
  free(mins);
  free(buf.w);
}

/* ------------------------------------------------------------ operator */
enum { O_XAT, O_XAM, O_XDT, O_XDM, O_ZBT, O_ZBM, O_X3D, O_YAT, O_Y2AT, O_YAM };

typedef struct orc_op {
  int kind, L, s1, s2, bc, cen, nlead, rotf, sym, mphys_bc, ltype;
  double bj, k, k2, h, nf;
  int64_t* swp; /* two-layer reduced: index of the layer-swapped orbit */
  double b1[2], b2[2], b3[2], b2b[4], b2c[16];
  int64_t nstate, n;
  double* tvec;
  table_t tab;
} orc_op;

/* XATMatVecProd2D::genTvec (TMat/tmat.hpp:208-310) */
static double gen_tvec_xat(double bj, double k, double h, int L, int bc, st_t s) {
  st_t mask = (1ull << L) - 1, a, b;
  int n1, n2, n0 = popc(s);
  double J1 = -bj, J2 = bj * k, hJ = -bj * h, bz1, bz2, bz0;
  switch (bc) {
    case 0:
      a = rotr(s, L, 1);
      b = rotr(s, L, 2);
      n1 = nanti2(s, a);
      n2 = nanti2(s, b);
      bz1 = bzexpn(L, n1, J1);
      bz2 = bzexpn(L, n2, J2);
      break;
    case 1:
      a = s >> 1;
      b = s >> 2;
      n1 = nanti2(s & mask >> 1, a);
      n2 = nanti2(s & mask >> 2, b);
      bz1 = bzexpn(L - 1, n1, J1);
      bz2 = bzexpn(L - 2, n2, J2);
      break;
    case 5:
    case 9:
      a = s << 1 | (bc == 9 ? 1 : 0);
      b = s >> 1;
      n1 = nanti2(s, a);
      n2 = nanti2(a & mask, b);
      bz1 = bzexpn(L + 1, n1, J1);
      bz2 = bzexpn(L, n2, J2);
      break;
    default: /* 13, 17 */
      a = s << 1 | (bc == 17 ? 1 : 0);
      b = s << 2 | (bc == 17 ? 3 : 0);
      n1 = nanti2(s, a);
      n2 = nanti2(s, b);
      bz1 = bzexpn(L + 1, n1, J1);
      bz2 = bzexpn(L + 2, n2, J2);
      break;
  }
  bz0 = bzexpn(L, n0, hJ);
  return exp(bz1 + bz2 + bz0);
}

/* XDTMatVecProd2D::genTvec (TMat/tmat.hpp:437-504) */
static double gen_tvec_xdt(double bj, double h, int L, int bc, st_t s) {
  int n1, n0 = popc(s), ns1 = L;
  double J1 = -bj, hJ = -bj * h;
  switch (bc) {
    case 0: n1 = nanti2(s, rotr(s, L, 1)); break;
    case 1: n1 = nanti2(s & (((1ull << L) - 1) >> 1), s >> 1); ns1 = L - 1; break;
    case 5: n1 = nanti2(s << 1, s); ns1 = L + 1; break;
    default: n1 = nanti2(s << 1 | 1, s); ns1 = L + 1; break;
  }
  return exp(bzexpn(ns1, n1, J1) + bzexpn(L, n0, hJ));
}

static void set_nf(orc_op* o) {
  double k = o->k, k2 = o->k2, bj = o->bj;
  int L = o->L;
  double nfe;
  switch (o->kind) {
    case O_XAT: o->nf = k < 0.5 ? exp(L * bj * (k - 2.0)) : exp(-L * bj * (k + 1.0)); break;
    case O_XAM: nfe = k < 0.5 ? L * (k - 2.0) : -L * (k + 1.0); o->nf = exp(bj * nfe); break;
    case O_XDT: o->nf = k < 0.5 ? exp(L * bj * 2.0 * (k - 1.0)) : exp(-L * bj * 2.0 * k); break;
    case O_XDM: nfe = k < 0.5 ? L * 2.0 * (k - 1.0) : -L * 2.0 * k; o->nf = exp(bj * nfe); break;
    case O_X3D: nfe = k < 0.5 ? L * (k - 3.0) : -L * (k + 2.0); o->nf = exp(bj * nfe); break;
    case O_YAT: o->nf = k < 0.5 ? exp(L * bj * (k - 2.0)) : exp(-L * bj * (k + 1.0)); break;
    case O_Y2AT: o->nf = k < 0.5 ? exp(2 * L * bj * (k - 2.0)) : exp(-2 * L * bj * (k + 1.0)); break;
    default: break;
  }
}

/* normfactor exponent of the diagonal BNNNI operators (TMat/tmat.cpp:491-511) */
static double zb_nfexp(double k, double k2, int L) {
  if (k + k2 < 0.5) return L * 2.0 * (k + k2 - 1.0);
  if (k < 0.5 && k2 - k < 0.5) return -L;
  if (k2 < 2 * k) return -L * 2.0 * k;
  return L * 2.0 * (k - k2);
}

static void make_bz(orc_op* o) {
  o->b1[0] = exp(o->bj);
  o->b1[1] = 1.0 / o->b1[0];
  o->b2[0] = exp(-o->bj * o->k);
  o->b2[1] = 1.0 / o->b2[0];
  o->b3[0] = exp(-o->bj * o->k2);
  o->b3[1] = 1.0 / o->b3[0];
  /* ZBM tables, TMat/tmatreduce.cpp:1415-1423 */
  o->b2b[0] = exp(-2 * o->bj * o->k);
  o->b2b[3] = 1.0 / o->b2b[0];
  o->b2b[1] = o->b2b[2] = 1.0;
  for (int r = 0; r < 16; ++r) {
    int ra = r >> 2, rb = r & 3;
    o->b2c[r] = exp(o->bj * (o->k * bzexp1(ra, 2) + o->k2 * bzexp1(rb, 2)));
  }
}

orc_op* orc_create(char model, int dim, int ax, int ec, double bj, double k, double k2, double h, int size) {
  orc_op* o = (orc_op*)calloc(1, sizeof(orc_op));
  o->bj = bj;
  o->k = k;
  o->k2 = k2;
  o->h = h;
  o->sym = 1;
  if (dim == 3) {
    o->s1 = size >> 16;
    o->s2 = size & 0xffff;
    o->L = o->s1 * o->s2;
  } else {
    o->L = size;
  }
  int L = o->L;
  o->nstate = 1ll << L;
  const int h0 = (h == 0.0);
  /* dispatch: TMat/pfunc.cpp:16-106 */
  if (model == 'A' && dim == 2) {
    if (ax == 1 || ax == 9 || ax == 17 || ax == 18 || ax == 19 || ax == 20) {
      o->kind = O_XAT;
      o->bc = ax == 1 ? 0 : ax == 9 ? 1 : ax == 17 ? 5 : ax == 18 ? 9 : ax == 19 ? 13 : 17;
    } else if (ax == 5 || ax == 13) {
      o->kind = O_XAM;
      int e = ax == 13 ? (ec | 1) : ec;
      o->bc = e & 1;
      o->cen = h0 && !(e & 2);
    } else if (ax == 0 || ax == 2) {
      o->kind = ax == 0 ? O_Y2AT : O_YAT;
      o->sym = 0;
    } else if (ax == 6) {
      o->kind = O_YAM;
      o->cen = h0 && !(ec & 2);
      o->sym = 0;
    } else {
      free(o);
      return NULL;
    }
  } else if (model == 'A' && dim == 3 && ax == 1) {
    o->kind = O_X3D;
    o->cen = h0;
    o->rotf = (k == 0.0) && o->s1 == o->s2;
  } else if (model == 'D') {
    if (ax == 1 || ax == 2 || ax == 17 || ax == 18) {
      o->kind = O_XDT;
      o->bc = (ax == 17) ? 5 : (ax == 18) ? 9 : 0;
    } else if (ax == 5 || ax == 6) {
      o->kind = O_XDM;
      o->cen = h0 && !(ec & 2);
    } else {
      free(o);
      return NULL;
    }
  } else if (model == 'B') {
    if (ax == 3) {
      o->kind = O_ZBT;
    } else if (ax == 7) {
      o->kind = O_ZBM;
      o->cen = h0 && !(ec & 2);
    } else if (ax == 6) {
      o->kind = O_YAM;
      o->ltype = 1;
      o->cen = h0 && !(ec & 2);
    } else {
      free(o);
      return NULL;
    }
    o->sym = 0;
  } else {
    free(o);
    return NULL;
  }
  make_bz(o);
  set_nf(o);
  switch (o->kind) {
    case O_XAT:
      o->n = o->nstate;
      o->mphys_bc = o->bc;
      o->tvec = (double*)malloc(o->n * 8);
#pragma omp parallel for
      for (int64_t s = 0; s < o->n; ++s) o->tvec[s] = gen_tvec_xat(0.5 * bj, k, h, L, o->bc, (st_t)s);
      break;
    case O_XDT:
      o->n = o->nstate;
      o->tvec = (double*)malloc(o->n * 8);
#pragma omp parallel for
      for (int64_t s = 0; s < o->n; ++s) o->tvec[s] = gen_tvec_xdt(0.5 * bj, h, L, o->bc, (st_t)s);
      break;
    case O_ZBT: {
      /* TMat/tmat.cpp:480-518 */
      double nfe = zb_nfexp(k, k2, L);
      double half = exp(0.5 * bj * nfe);
      o->nf = half * half;
      o->n = o->nstate;
      o->tvec = (double*)malloc(o->n * 8);
      double J1 = -0.5 * bj, J3 = k2 * 0.5 * bj, hJ = -0.5 * bj * h;
#pragma omp parallel for
      for (int64_t i = 0; i < o->n; ++i) {
        st_t s = (st_t)i;
        int n1 = nanti2(s, rotr(s, L, 1)), n2 = nanti2(s, rotr(s, L, 2)), n0 = popc(s);
        o->tvec[i] = exp(bzexpn(L, n1, J1) + bzexpn(L, n2, J3) + bzexpn(L, n0, hJ)) * half;
      }
      break;
    }
    case O_XAM: {
      /* TMat/tmatreduce.cpp:338-404 */
      o->mphys_bc = o->bc;
      o->nlead = (L < 10 || o->bc) ? 1 : 2 + (int)log2((double)L);
      double nfe = k < 0.5 ? L * (k - 2.0) : -L * (k + 1.0);
      gen_x2d(L, o->bc, o->cen, &o->tab);
      o->n = o->tab.n;
      o->tvec = (double*)malloc(o->n * 8);
      double hb = 0.5 * bj, J1 = -hb, J2 = hb * k, hJ = -hb * h, Jn = hb * nfe;
      st_t mask = o->nstate - 1;
#pragma omp parallel for
      for (int64_t r = 0; r < o->n; ++r) {
        st_t s = o->tab.idx[r];
        int n1, n2;
        if (!o->bc) {
          n1 = nanti2(s, rotr(s, L, 1));
          n2 = nanti2(s, rotr(s, L, 2));
        } else {
          n1 = nanti2(s & mask >> 1, s >> 1);
          n2 = nanti2(s & mask >> 2, s >> 2);
        }
        int n0 = popc(s);
        double bz = J1 * (2 * n1 - L) + J2 * (2 * n2 - L) + hJ * (2 * n0 - L) + Jn;
        o->tvec[r] = exp(bz) / sqrt((double)o->tab.dup[r]);
      }
      break;
    }
    case O_XDM: {
      /* TMat/tmatreduce.cpp:1024-1053, 1367-1400 */
      o->nlead = L < 10 ? 1 : 2 + (int)log2((double)L);
      double nfe = k < 0.5 ? L * 2.0 * (k - 1.0) : -L * 2.0 * k;
      gen_x2d(L, 0, o->cen, &o->tab);
      o->n = o->tab.n;
      o->tvec = (double*)malloc(o->n * 8);
      double hb = 0.5 * bj, J1 = -hb, hJ = -hb * h, Jn = hb * nfe;
      for (int64_t r = 0; r < o->n; ++r) {
        st_t s = o->tab.idx[r];
        int n1 = nanti2(s, rotr(s, L, 1)), n0 = popc(s);
        o->tvec[r] = exp(J1 * (2 * n1 - L) + hJ * (2 * n0 - L) + Jn) / sqrt((double)o->tab.dup[r]);
      }
      break;
    }
    case O_ZBM: {
      /* TMat/tmatreduce.cpp:1403-1454, 1813-1855 */
      o->nlead = L < 10 ? 2 : 2 + ((int)log2((double)L) & ~1);
      double nfe = zb_nfexp(k, k2, L);
      o->nf = exp(bj * nfe);
      gen_z2d(L, o->cen, &o->tab);
      o->n = o->tab.n;
      o->tvec = (double*)malloc(o->n * 8);
      double hb = 0.5 * bj, J1 = -hb, J3 = hb * k2, hJ = -hb * h, Jn = hb * nfe;
#pragma omp parallel for
      for (int64_t r = 0; r < o->n; ++r) {
        st_t s = o->tab.idx[r];
        int n1 = nanti2(s, rotr(s, L, 1)), n2 = nanti2(s, rotr(s, L, 2)), n0 = popc(s);
        double bz1 = bzexpn(L, n1, J1), bz2 = bzexpn(L, n2, J3), bz0 = bzexpn(L, n0, hJ);
        o->tvec[r] = exp(bz1 + bz2 + bz0 + Jn) / sqrt((double)o->tab.dup[r]);
      }
      break;
    }
    case O_X3D: {
      /* TMat/tmat3d.cpp:102-134, 179-201 */
      o->nlead = L < 10 ? 1 : 2 + (int)log2((double)L);
      double nfe = k < 0.5 ? L * (k - 3.0) : -L * (k + 2.0);
      gen_x3d(o->s1, o->s2, o->cen, o->rotf, &o->tab);
      o->n = o->tab.n;
      o->tvec = (double*)malloc(o->n * 8);
      double hb = 0.5 * bj, J1 = -hb, J2 = hb * k, hJ = -hb * h, Jn = hb * nfe;
#pragma omp parallel for
      for (int64_t r = 0; r < o->n; ++r) {
        st_t s = o->tab.idx[r];
        int n1a = nanti2(s, rff3(s, o->s1, o->s2, 1)), n1b = nanti2(s, dff3(s, o->s1, o->s2, 1));
        int n2 = nanti2(s, rff3(s, o->s1, o->s2, 2)), n0 = popc(s);
        double bz = 2 * J1 * (n1a + n1b - L) + J2 * (2 * n2 - L) + hJ * (2 * n0 - L) + Jn;
        o->tvec[r] = exp(bz) / sqrt((double)o->tab.dup[r]);
      }
      break;
    }
    case O_YAT: {
      /* YATMatVecProd2D::genTvec (TMat/tmat.hpp:361-366): the dense NN-only
       * x-ANNNI matrix (TMat/tmat.cpp:668-684) flattened column-major: entry
       * (row, col) = (low layer, high layer) */
      o->nstate = 1ll << (2 * L);
      o->n = o->nstate;
      o->tvec = (double*)malloc(o->n * 8);
      st_t mask = (1ull << L) - 1;
#pragma omp parallel for
      for (int64_t i = 0; i < o->n; ++i) {
        st_t row = (st_t)i & mask, col = (st_t)i >> L;
        o->tvec[i] = gen_tvec_xat(bj, 0.0, h, L, 0, row) * exp(bzexpn(L, nanti2(row, col), -bj));
      }
      break;
    }
    case O_Y2AT: {
      /* Y2ATMatVecProd2D::genTvec (TMat/tmat.hpp:396-414), Tv^(1/2) */
      o->nstate = 1ll << (2 * L);
      o->n = o->nstate;
      o->tvec = (double*)malloc(o->n * 8);
      st_t mask = (1ull << L) - 1;
      double J1 = -0.5 * bj, hJ = -0.5 * bj * h;
      o->b2[0] = exp(-2.0 * bj * k);
      o->b2[1] = 1.0 / o->b2[0];
#pragma omp parallel for
      for (int64_t i = 0; i < o->n; ++i) {
        st_t lo = (st_t)i & mask, hi = (st_t)i >> L;
        int n1 = nanti2(lo, rotr(lo, L, 1)), n2 = nanti2(hi, rotr(hi, L, 1)), n0 = nanti2(lo, hi);
        int fa = 2 * (n1 + n2 + n0) - 3 * L, fb = 2 * (popc((st_t)i) - L);
        o->tvec[i] = exp(J1 * fa + hJ * fb);
      }
      break;
    }
    case O_YAM: {
      /* YAMMatVecProd2D ctor / genTvec / genTvec1 (TMat/tmatreduce.cpp:663-797);
       * YBMMatVecProd2D is the layertype-1 form (:1018-1021) */
      o->nstate = 1ll << (2 * L);
      double nfe = o->ltype ? zb_nfexp(k, k2, L) : (k < 0.5 ? L * (k - 2.0) : -L * (k + 1.0));
      o->nf = exp(bj * nfe);
      gen_y2d(L, o->cen, &o->tab, &o->swp);
      o->n = o->tab.n;
      o->tvec = (double*)malloc(o->n * 8);
      st_t mask = (1ull << L) - 1;
      double hb = 0.5 * bj, J1 = -hb, hJ = -hb * h, Jn = hb * nfe, k1J = hb * k, k2J = hb * k2;
#pragma omp parallel for
      for (int64_t r = 0; r < o->n; ++r) {
        st_t s = o->tab.idx[r], l = s >> L, rt = s & mask;
        int n1 = nanti2(l, rotr(l, L, 1)), n2 = nanti2(l, rt), n0 = popc(l);
        double bz = J1 * (2 * (n1 + n2 - L)) + hJ * (2 * n0 - L) + Jn;
        if (o->ltype) {
          int b1 = nanti2(l, rotr(l, L, 2)), d1 = nanti2(l, rotr(rt, L, 1)), d2 = nanti2(l, rotl(rt, L, 1));
          bz += k1J * (2 * b1 - L) + k2J * (2 * (d1 + d2 - L));
        }
        o->tvec[r] = exp(bz) / sqrt((double)o->tab.dup[r]);
      }
      break;
    }
  }
  return o;
}

void orc_destroy(orc_op* o) {
  if (!o) return;
  free(o->tvec);
  free(o->tab.idx);
  free(o->tab.dup);
  free(o->swp);
  free(o);
}
int64_t orc_rows(const orc_op* o) { return o->n; }
double orc_normfactor(const orc_op* o) { return o->nf; }
int orc_symmetric(const orc_op* o) { return o->sym; }
int orc_layer_size(const orc_op* o) { return o->L; }

int64_t orc_orbit(const orc_op* o, uint64_t* idx, uint16_t* dup) {
  if (!o->tab.n) return -1;
  if (idx) memcpy(idx, o->tab.idx, o->tab.n * 8);
  if (dup) memcpy(dup, o->tab.dup, o->tab.n * 2);
  return o->tab.n;
}

/* ------------------------------------------------------------ full ops */
/* in-place butterfly over the low nbits of a length-2^nbits vector
 * (XATMatVecProd2D::perform_op inner loops, TMat/tmat.cpp:80-93;
 * XAMMatVecProd2D::permute_mult_TL, TMat/tmatreduce.cpp:546-563) */
static void bfly(const double* b1, double* y, int64_t len, int nbits) {
  for (int it = 0; it < nbits; ++it) {
    st_t m = 1ull << it;
#pragma omp parallel for
    for (int64_t r = 0; r < len; ++r) {
      if ((st_t)r & m) {
        double d = y[r];
        y[r] = b1[0] * d + b1[1] * y[r ^ m];
        y[r ^ m] = b1[1] * d + b1[0] * y[r ^ m];
      }
    }
  }
}

/* XATMatVecProd2D::perform_op, TMat/tmat.cpp:71-102 */
static void op_xat(const orc_op* o, const double* x, double* y) {
  int64_t n = o->n;
#pragma omp parallel for
  for (int64_t r = 0; r < n; ++r) y[r] = o->tvec[r] * x[r];
  bfly(o->b1, y, n, o->L);
#pragma omp parallel for
  for (int64_t r = 0; r < n; ++r) y[r] = o->nf * o->tvec[r] * y[r];
}

/* XDTMatVecProd2D::permute_mult_T1(_last), TMat/tmat.cpp:344-376 */
static void xdt_step(const orc_op* o, const double* xin, double* yout, int last, st_t lastbit) {
  const int L = o->L;
  st_t nst = o->nstate, nb = nst << 1, mask = nst - 1, maskb = nst - 2;
#pragma omp parallel for
  for (int64_t i = 0; i < (int64_t)nb; ++i) {
    st_t rpb = (st_t)i, aux = rpb >> L, rp = rpb & mask;
    st_t rpp = aux << L | rotr(rp, L, 1);
    st_t rq = (rp & maskb) | aux, sb = rp & 1;
    st_t nb2 = last ? lastbit : ((rq >> 1) & 1);
    yout[rpp] = o->b1[sb ^ aux] * o->b2[nb2 ^ sb] * (o->b2[sb] * xin[rq] + o->b2[sb ^ 1] * xin[rq | nst]);
  }
}

/* XDTMatVecProd2D::perform_op, TMat/tmat.cpp:379-476 */
static void op_xdt(const orc_op* o, const double* x, double* y) {
  const int L = o->L;
  st_t nst = o->nstate, nc = nst >> 1;
  double* t1 = (double*)malloc(nst * 2 * 8);
  double* t2 = (double*)malloc(nst * 2 * 8);
  if (o->bc == 0) {
    for (st_t lb = 0; lb < 2; ++lb) {
      double *p1 = t1, *p2 = t2, *sw;
#pragma omp parallel for
      for (int64_t i = 0; i < (int64_t)nst; ++i) {
        st_t rp = (st_t)i, rpb = (rp & nc) << 1 | rp;
        p1[rpb] = ((rp & 1) == lb) ? o->tvec[rp] * x[rp] : 0.0;
        p1[rpb ^ nst] = 0.0;
      }
      for (int r = 0; r < L - 1; ++r) {
        xdt_step(o, p1, p2, 0, 0);
        sw = p1;
        p1 = p2;
        p2 = sw;
      }
      xdt_step(o, p1, p2, 1, lb);
#pragma omp parallel for
      for (int64_t i = 0; i < (int64_t)nst; ++i) {
        double v = o->nf * o->tvec[i] * (p2[i] + p2[(st_t)i ^ nst]);
        if (lb == 0)
          y[i] = v;
        else
          y[i] += v;
      }
    }
  } else {
    double *p1 = t1, *p2 = t2, *sw;
#pragma omp parallel for
    for (int64_t i = 0; i < (int64_t)nst; ++i) {
      st_t rp = (st_t)i;
      if (o->bc == 5) {
        p1[rp] = o->tvec[rp] * x[rp] * o->b2[rp & 1] * o->b2[rp >> (L - 1)];
        p1[rp | nst] = 0.0;
      } else {
        p1[rp | nst] = o->tvec[rp] * x[rp] * o->b2[(rp & 1) ^ 1] * o->b2[rp >> (L - 1)];
        p1[rp] = 0.0;
      }
    }
    for (int r = 0; r < L - 1; ++r) {
      xdt_step(o, p1, p2, 0, 0);
      sw = p1;
      p1 = p2;
      p2 = sw;
    }
    xdt_step(o, p1, p2, 1, 0);
#pragma omp parallel for
    for (int64_t i = 0; i < (int64_t)nst; ++i) y[i] = o->nf * o->tvec[i] * (p2[i] + p2[(st_t)i | nst]);
  }
  free(t1);
  free(t2);
}

/* ZBTMatVecProd2D::permute_mult_T1(_last), TMat/tmat.cpp:521-588 */
static void zbt_step(const orc_op* o, const double* xin, double* yout, int last, st_t lastbit, int dir) {
  const int L = o->L;
  st_t nst = o->nstate, nb = nst << 2, mask = nst - 1, maskb = nst - 4;
  const double *b1 = o->b1, *b2 = o->b2, *b3 = o->b3;
#pragma omp parallel for
  for (int64_t i = 0; i < (int64_t)nb; ++i) {
    st_t rpb = (st_t)i, aux = rpb >> L, rp = rpb & mask;
    st_t rpp = aux << L | rotr(rp, L, 2);
    st_t rq = (rp & maskb) | aux;
    st_t sl = rp >> 1 & 1, sr = rp & 1, pl = aux >> 1, pr = aux & 1;
    st_t fl = last ? lastbit >> 1 : (rp >> 3 & 1), fr = last ? (lastbit & 1) : (rp >> 2 & 1);
    double v;
    if (!dir)
      v = b1[sr ^ pl] * b2[sr ^ fr] * b2[sl ^ fl] * b3[sr ^ pr] * b3[sl ^ pl];
    else
      v = b1[sl ^ fr] * b1[sl ^ pr] * b2[sr ^ fr] * b2[sl ^ fl] * b3[sr ^ pr] * b3[sl ^ pl];
    double d = 0.0;
    for (st_t q = 0; q < 4; ++q) {
      st_t al = q >> 1, ar = q & 1, rqq = q << L | rq;
      if (!dir)
        d += xin[rqq] * b1[sr ^ al] * b2[sr ^ ar] * b2[sl ^ al];
      else
        d += xin[rqq] * b2[sr ^ ar] * b2[sl ^ al];
    }
    yout[rpp] = v * d;
  }
}

/* ZBTMatVecProd2D::perform_op_internal, TMat/tmat.cpp:596-649 */
static void op_zbt(const orc_op* o, const double* x, double* y, int dir) {
  const int L = o->L;
  st_t nst = o->nstate, nc = nst >> 1 | nst >> 2;
  double* t1 = (double*)malloc(nst * 4 * 8);
  double* t2 = (double*)malloc(nst * 4 * 8);
  for (st_t lb = 0; lb < 4; ++lb) {
    double *p1 = t1, *p2 = t2, *sw;
#pragma omp parallel for
    for (int64_t i = 0; i < (int64_t)nst; ++i) {
      st_t rp = (st_t)i, rpb = (rp & nc) << 2 | rp;
      p1[rpb] = ((rp & 3) == lb) ? o->tvec[rp] * x[rp] : 0.0;
      p1[rpb ^ nst] = p1[rpb ^ (nst << 1)] = p1[rpb ^ (nc << 2)] = 0.0;
    }
    for (int r = 0; r < L / 2 - 1; ++r) {
      zbt_step(o, p1, p2, 0, 0, dir);
      sw = p1;
      p1 = p2;
      p2 = sw;
    }
    zbt_step(o, p1, p2, 1, lb, dir);
#pragma omp parallel for
    for (int64_t i = 0; i < (int64_t)nst; ++i) {
      st_t rp = (st_t)i;
      double v = o->tvec[rp] * (p2[rp] + p2[rp ^ nst] + p2[rp ^ (nst << 1)] + p2[rp ^ (nc << 2)]);
      if (lb == 0)
        y[i] = v;
      else
        y[i] += v;
    }
  }
  free(t1);
  free(t2);
}

/* ------------------------------------------------------------ reduced ops */
/* XAMMatVecProd2D::perform_op, TMat/tmatreduce.cpp:406-529 */
static void op_xam(const orc_op* o, const double* x, double* y) {
  const int L = o->L, nl = o->nlead, nsub = L - nl;
  st_t nst = o->nstate, nloop = 1ull << nl, vsz = nst >> nl;
  st_t mb = vsz - 1, mc = nloop - 1, mbinv = ~mb & (nst - 1);
  double* yt = (double*)malloc(vsz * 8);
  const int64_t R = o->n;
  if (o->cen) nloop >>= 1;
  for (st_t rd = 0; rd < nloop; ++rd) {
    st_t rdh = rd << nsub, rdr = brev(rd, nl);
#pragma omp parallel for
    for (int64_t r = 0; r < R; ++r) {
      double d = o->tvec[r] * x[r];
      st_t s0 = o->tab.idx[r], ns = s0;
      if (o->bc) {
        if ((ns & mbinv) == rdh)
          yt[ns & mb] = d;
        else if (o->cen && (~ns & mbinv) == rdh)
          yt[~ns & mb] = d;
        if ((ns & mc) == rdr)
          yt[brev(ns, L) & mb] = d;
        else if (o->cen && (~ns & mc) == rdr)
          yt[brev(~ns, L) & mb] = d;
      } else {
        do {
          if ((ns & mbinv) == rdh)
            yt[ns & mb] = d;
          else if (o->cen && (~ns & mbinv) == rdh)
            yt[~ns & mb] = d;
          if ((ns & mc) == rdr)
            yt[brev(ns, L) & mb] = d;
          else if (o->cen && (~ns & mc) == rdr)
            yt[brev(~ns, L) & mb] = d;
          ns = ns >> 1 | (ns & 1) << (L - 1);
        } while (ns != s0);
      }
    }
    bfly(o->b1, yt, (int64_t)vsz, nsub);
#pragma omp parallel for
    for (int64_t r = 0; r < R; ++r) {
      st_t s = o->tab.idx[r];
      double d = powdi(o->b1, bzexp2(s >> nsub, rd, nl));
      double v = o->cen ? d * yt[s & mb] + yt[~s & mb] / d : d * yt[s & mb];
      if (rd)
        y[r] += v;
      else
        y[r] = v;
    }
  }
#pragma omp parallel for
  for (int64_t r = 0; r < R; ++r) y[r] *= o->tab.dup[r] * o->tvec[r];
  free(yt);
}

/* XAMMatVecProd3D::perform_op, TMat/tmat3d.cpp:203-321 */
static void op_x3d(const orc_op* o, const double* x, double* y) {
  const int L = o->L, nl = o->nlead, nsub = L - nl, s1 = o->s1, s2 = o->s2;
  st_t nst = o->nstate, nloop = 1ull << nl, vsz = nst >> nl;
  st_t mask = nst - 1, mb = vsz - 1, mbinv = ~mb & (nst - 1);
  double* yt = (double*)malloc(vsz * 8);
  const int64_t R = o->n;
  if (o->cen) nloop >>= 1;
  for (st_t rd = 0; rd < nloop; ++rd) {
    st_t rdh = rd << nsub;
#pragma omp parallel for
    for (int64_t r = 0; r < R; ++r) {
      double d = o->tvec[r] * x[r];
      st_t s = o->tab.idx[r];
      for (int rr = 0; rr <= o->rotf; ++rr) {
        st_t a = rr ? rot3(s, s1) : s;
        for (int c = 0; c <= o->cen; ++c) {
          st_t b = c ? (~a & mask) : a;
          for (int m1 = 0; m1 < 2; ++m1) {
            st_t e = m1 ? refl3(b, s1, s2, 0) : b;
            for (int m2 = 0; m2 < 2; ++m2) {
              st_t f = m2 ? refl3(e, s1, s2, 1) : e;
              st_t o1 = f;
              do {
                st_t o2 = o1;
                do {
                  if ((o2 & mbinv) == rdh) yt[o2 & mb] = d;
                  o2 = dff3(o2, s1, s2, 1);
                } while (o2 != o1);
                o1 = rff3(o1, s1, s2, 1);
              } while (o1 != f);
            }
          }
        }
      }
    }
    bfly(o->b1, yt, (int64_t)vsz, nsub);
#pragma omp parallel for
    for (int64_t r = 0; r < R; ++r) {
      st_t s = o->tab.idx[r];
      double d = powdi(o->b1, bzexp2(s >> nsub, rd, nl));
      double v = o->cen ? d * yt[s & mb] + yt[~s & mb] / d : d * yt[s & mb];
      if (rd)
        y[r] += v;
      else
        y[r] = v;
    }
  }
#pragma omp parallel for
  for (int64_t r = 0; r < R; ++r) y[r] *= o->tab.dup[r] * o->tvec[r];
  free(yt);
}

/* XDMMatVecProd2D::permute_mult_TL, TMat/tmatreduce.cpp:1230-1259 */
static void xdm_sweep(const orc_op* o, double* yt, int outbit) {
  const int nl = o->nlead, nlp = o->L - nl;
  st_t part = o->nstate >> nl;
  const double *b1 = o->b1, *b2 = o->b2;
  for (int it = 0; it < nlp; ++it) {
    st_t m = 1ull << it, bs = ~m & (o->nstate - 1);
#pragma omp parallel for
    for (int64_t i = 0; i < (int64_t)part; ++i) {
      st_t rp = (st_t)i;
      if (!(rp & m)) continue;
      int nb = outbit;
      if (it < nlp - 1) nb = (rp >> (it + 1)) & 1;
      st_t i00 = rp & bs, i01 = rp, i10 = (rp & bs) | part, i11 = rp | part;
      double d00 = yt[i00], d01 = yt[i01], d10 = yt[i10], d11 = yt[i11];
      yt[i00] = b1[0] * b2[nb] * (b2[0] * d00 + b2[1] * d10);
      yt[i01] = b1[1] * b2[nb ^ 1] * (b2[1] * d00 + b2[0] * d10);
      yt[i10] = b1[1] * b2[nb] * (b2[0] * d01 + b2[1] * d11);
      yt[i11] = b1[0] * b2[nb ^ 1] * (b2[1] * d01 + b2[0] * d11);
    }
  }
}

/* XDMMatVecProd2D::perform_op, TMat/tmatreduce.cpp:1055-1228 */
static void op_xdm(const orc_op* o, const double* x, double* y) {
  const int L = o->L, nl = o->nlead, nsub = L - nl;
  st_t nst = o->nstate, nloop = 1ull << nl, vsz = nst >> nl;
  st_t mask = nst - 1, mb = vsz - 1, mc = nloop - 1, md = mc >> 1, mbinv = ~mb & (nst - 1);
  st_t nsubst = 1ull << nsub;
  double* xt = (double*)malloc(vsz * 8);
  double* yt = (double*)malloc(2 * vsz * 8);
  const int64_t R = o->n;
  for (int64_t r = 0; r < R; ++r) y[r] = 0.0;
  if (o->cen) nloop >>= 1;
  for (st_t rd = 0; rd < nloop; ++rd) {
    st_t rdh = rd << nsub, rdr = brev(rd, nl);
#pragma omp parallel for
    for (int64_t r = 0; r < R; ++r) {
      double d = o->tvec[r] * x[r];
      st_t s0 = o->tab.idx[r], ns = s0;
      do {
        if ((ns & mbinv) == rdh)
          xt[ns & mb] = d;
        else if (o->cen && (~ns & mbinv) == rdh)
          xt[~ns & mb] = d;
        if ((ns & mc) == rdr)
          xt[brev(ns, L) & mb] = d;
        else if (o->cen && (~ns & mc) == rdr)
          xt[brev(~ns, L) & mb] = d;
        ns = ns >> 1 | (ns & 1) << (L - 1);
      } while (ns != s0);
    }
    for (int fb = 0; fb < 2; ++fb) {
      st_t gbit = o->cen ? 0 : (rd >> (nl - 1) << nsub);
#pragma omp parallel for
      for (int64_t i = 0; i < (int64_t)vsz; ++i) {
        st_t rp = (st_t)i;
        yt[rp | gbit] = xt[rp] * o->b2[(rp & 1) ^ fb];
        yt[rp | (gbit ^ nsubst)] = 0.0;
      }
      xdm_sweep(o, yt, (int)(rd & 1));
#pragma omp parallel for
      for (int64_t r = 0; r < R; ++r) {
        st_t s = o->tab.idx[r];
        if (o->cen) {
          if (fb) s = ~s & mask;
        } else if ((s >> (L - 1)) ^ (st_t)fb) {
          continue;
        }
        st_t rdb = s >> nsub;
        double d = powdi(o->b1, bzexp2(rd, rdb, nl));
        d *= powdi(o->b2, bzexp1((rd >> 1 ^ rdb) & md, nl - 1) + bzexp1((rd ^ rdb >> 1) & md, nl - 1));
        y[r] += d * (yt[s & mb] * o->b2[rdb & 1] + yt[(s & mb) | vsz] * o->b2[(rdb & 1) ^ 1]);
      }
    }
  }
#pragma omp parallel for
  for (int64_t r = 0; r < R; ++r) y[r] *= o->tab.dup[r] * o->tvec[r];
  free(xt);
  free(yt);
}

/* ZBMMatVecProd2D::permute_mult_T1(_last), TMat/tmatreduce.cpp:1620-1706 */
static void zbm_step(const orc_op* o, const double* xin, double* yout, int last, st_t lastbit, int dir) {
  const int nsub = o->L - o->nlead;
  st_t vsz = o->nstate >> o->nlead, nb = vsz << 2, maskb = vsz - 4;
  const double *b1 = o->b1, *b2b = o->b2b, *b2c = o->b2c;
#pragma omp parallel for
  for (int64_t i = 0; i < (int64_t)nb; ++i) {
    st_t rpb = (st_t)i, aux = rpb & 3, rp = rpb >> 2;
    st_t rpp = rotr(rp, nsub, 2) << 2 | aux;
    st_t rq = ((rp & maskb) | aux) << 2;
    unsigned sb = (unsigned)(rp & 3);
    unsigned j2 = (unsigned)(((last ? (lastbit << 2) : (rp & 0xc)) | aux) ^ (sb << 2 | sb));
    double v, d;
    if (!dir) {
      unsigned sr = rp & 1, pl = (unsigned)(aux >> 1);
      v = b1[sr ^ pl] * b2c[j2];
      d = xin[rq] * b1[sr] * b2b[sb];
      d += xin[rq + 1] * b1[sr] * b2b[sb ^ 1];
      d += xin[rq + 2] * b1[sr ^ 1] * b2b[sb ^ 2];
      d += xin[rq + 3] * b1[sr ^ 1] * b2b[sb ^ 3];
    } else {
      unsigned sl = rp >> 1 & 1, fr = last ? (unsigned)(lastbit & 1) : (unsigned)(rp >> 2 & 1), pr = aux & 1;
      v = b1[sl ^ fr] * b1[sl ^ pr] * b2c[j2];
      d = xin[rq] * b2b[sb];
      d += xin[rq + 1] * b2b[sb ^ 1];
      d += xin[rq + 2] * b2b[sb ^ 2];
      d += xin[rq + 3] * b2b[sb ^ 3];
    }
    yout[rpp] = v * d;
  }
}

/* ZBMMatVecProd2D::leadingbz, TMat/tmatreduce.cpp:1708-1746 */
static double zbm_lead(const orc_op* o, const double* yt, st_t s, st_t lead, st_t lastbit, int dir) {
  const st_t EVEN = 0x5555555555555555ull;
  const int nl = o->nlead, nsub = o->L - nl;
  st_t vsz = o->nstate >> nl, mb = vsz - 1, mc = (1ull << nl) - 1, md = mc >> 2;
  st_t nlb = s >> nsub, nh = (s & mb) << 2;
  double f1 = powdi(o->b3, bzexp2(nlb, lead, nl));
  f1 *= powdi(o->b2, bzexp2(nlb, lead >> 2 | lastbit << (nl - 2), nl) + bzexp2(nlb >> 2, lead & md, nl - 2));
  st_t in, ix;
  int ii;
  double f2;
  if (!dir) {
    in = nlb & EVEN;
    in |= in >> 1;
    ix = (lead >> 1) & EVEN;
    ix |= (ix << 1) & (mc >> 1);
    ii = bzexp2(in, ix, nl - 1);
    unsigned lb = nlb & 1;
    f2 = o->b1[lb] * (o->b2b[nlb & 3] * yt[nh] + o->b2b[(nlb & 3) ^ 1] * yt[nh + 1]) +
         o->b1[lb ^ 1] * (o->b2b[(nlb & 3) ^ 2] * yt[nh + 2] + o->b2b[(nlb & 3) ^ 3] * yt[nh + 3]);
  } else {
    in = (nlb >> 1) & EVEN;
    in |= in << 1;
    ix = (lead | (lastbit << nl)) & EVEN;
    ix = (ix & mc) | (ix >> 1);
    ii = bzexp2(in, ix, nl);
    f2 = o->b2b[nlb & 3] * yt[nh] + o->b2b[(nlb & 3) ^ 1] * yt[nh + 1] + o->b2b[(nlb & 3) ^ 2] * yt[nh + 2] +
         o->b2b[(nlb & 3) ^ 3] * yt[nh + 3];
  }
  f1 *= powdi(o->b1, ii);
  return f1 * f2;
}

/* ZBMMatVecProd2D::perform_op_internal, TMat/tmatreduce.cpp:1461-1617 */
static void op_zbm(const orc_op* o, const double* x, double* y, int dir) {
  const int L = o->L, nl = o->nlead, nsub = L - nl;
  st_t nst = o->nstate, nloop = 1ull << nl, vsz = nst >> nl;
  st_t mask = nst - 1, mb = vsz - 1, mc = nloop - 1, mbinv = ~mb & (nst - 1);
  double* xt = (double*)malloc(vsz * 8);
  double* p1 = (double*)malloc(4 * vsz * 8);
  double* p2 = (double*)malloc(4 * vsz * 8);
  const int64_t R = o->n;
  for (int64_t r = 0; r < R; ++r) y[r] = 0.0;
  if (o->cen) nloop >>= 1;
  for (st_t rd = 0; rd < nloop; ++rd) {
    st_t rdh = rd << nsub, rdhi = (~rd & mc) << nsub;
#pragma omp parallel for
    for (int64_t r = 0; r < R; ++r) {
      double d = o->tvec[r] * x[r];
      st_t s0 = o->tab.idx[r], ns = s0;
      do {
        if ((ns & mbinv) == rdh)
          xt[ns & mb] = d;
        else if (o->cen && (ns & mbinv) == rdhi)
          xt[~ns & mb] = d;
        st_t is = brev(ns >> 1 | (ns & 1) << (L - 1), L);
        if ((is & mbinv) == rdh)
          xt[is & mb] = d;
        else if (o->cen && (is & mbinv) == rdhi)
          xt[~is & mb] = d;
        ns = ns >> 2 | (ns & 3) << (L - 2);
      } while (ns != s0);
    }
    st_t fbit = rd >> (nl - 2);
    for (st_t lb = 0; lb < 4; ++lb) {
      double *a = p1, *b = p2, *sw;
#pragma omp parallel for
      for (int64_t i = 0; i < (int64_t)vsz; ++i) {
        st_t rp = (st_t)i, rrp = rp << 2 | fbit;
        a[rrp] = ((rp & 3) == lb) ? xt[rp] : 0.0;
        a[rrp ^ 1] = a[rrp ^ 2] = a[rrp ^ 3] = 0.0;
      }
      for (int r = 0; r < nsub / 2 - 1; ++r) {
        zbm_step(o, a, b, 0, 0, dir);
        sw = a;
        a = b;
        b = sw;
      }
      zbm_step(o, a, b, 1, rd & 3, dir);
#pragma omp parallel for
      for (int64_t r = 0; r < R; ++r) {
        st_t s = o->tab.idx[r];
        double d = zbm_lead(o, b, s, rd, lb, dir);
        if (o->cen) d += zbm_lead(o, b, ~s & mask, rd, lb, dir);
        y[r] += d;
      }
    }
  }
#pragma omp parallel for
  for (int64_t r = 0; r < R; ++r) y[r] *= o->tab.dup[r] * o->tvec[r];
  free(xt);
  free(p1);
  free(p2);
}

/* ------------------------------------------------------------ dispatch */
/* in-place Kronecker of [[w0, w1], [w1, w0]] over bits [lo, lo+nb) of a
 * vector of 2^nbits entries (TMat/tmatreduce.cpp:806-824 per bit) */
static void kron_bits(double* v, int nbits, int lo, int nb, double w0, double w1) {
  const int64_t n = 1ll << nbits;
  for (int b = lo; b < lo + nb; ++b) {
    const int64_t m = 1ll << b;
#pragma omp parallel for if (n > 65536)
    for (int64_t i = 0; i < n; ++i) {
      if (i & m) continue;
      double a = v[i], c = v[i | m];
      v[i] = w0 * a + w1 * c;
      v[i | m] = w1 * a + w0 * c;
    }
  }
}

/* YATMatVecProd2D::perform_op (TMat/tmat.cpp:213-242): the L shift-and-mix
 * steps on the high layer amount to the Kronecker factor on the high L bits;
 * then y[s] = nf * Tvec[s] * v[swap(s)].  dir=1: YATMatVecProd2D_T
 * (TMat/tmat.cpp:141-173), the exact transpose: v = Kronecker on the low
 * bits of Tvec .* x, y[swap(s)] = nf * v[s]. */
static void op_yat(const orc_op* o, const double* x, double* y, int dir) {
  const int L = o->L;
  const int64_t n = o->n;
  double* v = (double*)malloc(n * 8);
  if (!dir) {
    memcpy(v, x, n * 8);
    kron_bits(v, 2 * L, L, L, o->b2[0], o->b2[1]);
#pragma omp parallel for
    for (int64_t i = 0; i < n; ++i) y[i] = o->nf * o->tvec[i] * v[y_swap((st_t)i, L)];
  } else {
#pragma omp parallel for
    for (int64_t i = 0; i < n; ++i) v[i] = o->tvec[i] * x[i];
    kron_bits(v, 2 * L, 0, L, o->b2[0], o->b2[1]);
#pragma omp parallel for
    for (int64_t i = 0; i < n; ++i) y[y_swap((st_t)i, L)] = o->nf * v[i];
  }
  free(v);
}

/* Y2ATMatVecProd2D::perform_op (TMat/tmat.cpp:292-307).  One step of
 * permute_mult_T1 (:275-289) mixes the bit pair (0, L) by a 4x4 matrix and
 * rotates both layers; over L steps every pair (i, L+i) gets the same 4x4
 * matrix once.  With p = (low bit a, high bit b), j = a^b:
 *   out(p) = w1[j] (w2[0] in(p) + in(p ^ high)) + w1[j^1] (w2[1] in(p ^ both) + in(p ^ low)). */
static void op_y2at(const orc_op* o, const double* x, double* y) {
  const int L = o->L;
  const int64_t n = o->n;
  double* v = (double*)malloc(n * 8);
#pragma omp parallel for
  for (int64_t i = 0; i < n; ++i) v[i] = o->tvec[i] * x[i];
  for (int b = 0; b < L; ++b) {
    const int64_t ml = 1ll << b, mh = 1ll << (L + b);
#pragma omp parallel for if (n > 65536)
    for (int64_t i = 0; i < n; ++i) {
      if (i & (ml | mh)) continue;
      double in[4], out[4];
      for (int q = 0; q < 4; ++q) in[q] = v[i | ((q & 1) ? ml : 0) | ((q & 2) ? mh : 0)];
      for (int p = 0; p < 4; ++p) {
        int a = p & 1, bb = p >> 1, j = a ^ bb;
        out[p] = o->b1[j] * (o->b2[0] * in[p] + in[p ^ 2]) + o->b1[j ^ 1] * (o->b2[1] * in[p ^ 3] + in[p ^ 1]);
      }
      for (int q = 0; q < 4; ++q) v[i | ((q & 1) ? ml : 0) | ((q & 2) ? mh : 0)] = out[q];
    }
  }
#pragma omp parallel for
  for (int64_t i = 0; i < n; ++i) y[i] = o->nf * o->tvec[i] * v[i];
  free(v);
}

/* YAMMatVecProd2D::perform_op (TMat/tmatreduce.cpp:827-876) and
 * YAMMatVecProd2D_T::perform_op (:953-1016).  Per block of representatives
 * sharing the left layer l: fill the right-layer vector at every image g(r)
 * with g in the stabiliser of l, apply the Kronecker factor on the L right
 * bits, and write each representative's entry to its layer-swapped orbit
 * (dir=0) or to itself reading the swapped input (dir=1). */
static void op_yam(const orc_op* o, const double* x, double* y, int dir) {
  const int L = o->L;
  const st_t mask = (1ull << L) - 1;
  const int64_t R = o->n;
  const int ng = 2 * L * (o->cen ? 2 : 1);
  /* block starts */
  int64_t nb = 0;
  int64_t* start = (int64_t*)malloc((R + 1) * sizeof(int64_t));
  for (int64_t r = 0; r < R; ++r)
    if (r == 0 || (o->tab.idx[r] >> L) != (o->tab.idx[r - 1] >> L)) start[nb++] = r;
  start[nb] = R;
#pragma omp parallel
  {
    double* tmp = (double*)malloc((1ull << L) * 8);
    int* stab = (int*)malloc(ng * sizeof(int));
#pragma omp for schedule(dynamic)
    for (int64_t bk = 0; bk < nb; ++bk) {
      const st_t l = o->tab.idx[start[bk]] >> L;
      int ns = 0;
      for (int g = 0; g < ng; ++g) {
        int sh = g % L, rf = (g / L) & 1, f = g / (2 * L);
        if ((y_act(l << L, L, sh, rf, f) >> L) == l) stab[ns++] = g;
      }
      for (int64_t r = start[bk]; r < start[bk + 1]; ++r) {
        int64_t src = dir ? o->swp[r] : r;
        double v = o->tvec[src] * x[src];
        st_t rt = o->tab.idx[r] & mask;
        for (int q = 0; q < ns; ++q) {
          int g = stab[q], sh = g % L, rf = (g / L) & 1, f = g / (2 * L);
          tmp[y_act(rt, L, sh, rf, f) & mask] = v;
        }
      }
      kron_bits(tmp, L, 0, L, o->b2[0], o->b2[1]);
      for (int64_t r = start[bk]; r < start[bk + 1]; ++r) {
        int64_t dst = dir ? r : o->swp[r];
        y[dst] = o->tvec[dst] * o->tab.dup[dst] * tmp[o->tab.idx[r] & mask];
      }
    }
    free(tmp);
    free(stab);
  }
  free(start);
}

void orc_perform_op(const orc_op* o, const double* x, double* y) {
  switch (o->kind) {
    case O_XAT: op_xat(o, x, y); break;
    case O_XAM: op_xam(o, x, y); break;
    case O_XDT: op_xdt(o, x, y); break;
    case O_XDM: op_xdm(o, x, y); break;
    case O_ZBT: op_zbt(o, x, y, 0); break;
    case O_ZBM: op_zbm(o, x, y, 0); break;
    case O_X3D: op_x3d(o, x, y); break;
    case O_YAT: op_yat(o, x, y, 0); break;
    case O_Y2AT: op_y2at(o, x, y); break;
    case O_YAM: op_yam(o, x, y, 0); break;
  }
}

/* transpose (ZBTMatVecProd2D_T / ZBMMatVecProd2D_T): optdirection = 1 */
int orc_perform_op_t(const orc_op* o, const double* x, double* y) {
  if (o->kind == O_ZBT) {
    op_zbt(o, x, y, 1);
    return 0;
  }
  if (o->kind == O_ZBM) {
    op_zbm(o, x, y, 1);
    return 0;
  }
  if (o->kind == O_YAT) {
    op_yat(o, x, y, 1);
    return 0;
  }
  if (o->kind == O_YAM) {
    op_yam(o, x, y, 1);
    return 0;
  }
  /* symmetric, or Y2ATMatVecProd2D whose get_t_instance is the operator
   * itself (TMat/tmat.hpp:382-384) */
  orc_perform_op(o, x, y);
  return 1;
}

/* time `reps` leading-bit slices of the reduced x-ANNNI product (bounded CPU
 * baseline sample at widths where one full product takes minutes); returns
 * the slices done.  y receives the partial sum. */
int64_t orc_xam_slices(const orc_op* o, const double* x, double* y, int64_t first, int64_t count) {
  if (o->kind != O_XAM) return -1;
  const int L = o->L, nl = o->nlead, nsub = L - nl;
  st_t nst = o->nstate, nloop = 1ull << nl, vsz = nst >> nl;
  st_t mb = vsz - 1, mc = nloop - 1, mbinv = ~mb & (nst - 1);
  double* yt = (double*)malloc(vsz * 8);
  const int64_t R = o->n;
  if (o->cen) nloop >>= 1;
  int64_t done = 0;
  for (st_t rd = (st_t)first; rd < nloop && done < count; ++rd, ++done) {
    st_t rdh = rd << nsub, rdr = brev(rd, nl);
#pragma omp parallel for schedule(static)
    for (int64_t r = 0; r < R; ++r) {
      double d = o->tvec[r] * x[r];
      st_t s0 = o->tab.idx[r], ns = s0;
      do {
        if ((ns & mbinv) == rdh)
          yt[ns & mb] = d;
        else if (o->cen && (~ns & mbinv) == rdh)
          yt[~ns & mb] = d;
        if ((ns & mc) == rdr)
          yt[brev(ns, L) & mb] = d;
        else if (o->cen && (~ns & mc) == rdr)
          yt[brev(~ns, L) & mb] = d;
        ns = ns >> 1 | (ns & 1) << (L - 1);
      } while (ns != s0);
    }
    bfly(o->b1, yt, (int64_t)vsz, nsub);
#pragma omp parallel for schedule(static)
    for (int64_t r = 0; r < R; ++r) {
      st_t s = o->tab.idx[r];
      double d = powdi(o->b1, bzexp2(s >> nsub, rd, nl));
      double v = o->cen ? d * yt[s & mb] + yt[~s & mb] / d : d * yt[s & mb];
      if (done)
        y[r] += v;
      else
        y[r] = v;
    }
  }
  free(yt);
  return done;
}
int64_t orc_xam_nslices(const orc_op* o) { return o->cen ? (1ll << o->nlead) / 2 : (1ll << o->nlead); }

/* ------------------------------------------------------------ observables */
/* moments: TMat/tmatphys.cpp:13-38, 108-135; TMat/tmatreduce.cpp:565-591,
 * 1261-1287, 1748-1775; TMat/tmat3d.cpp:137-163 */
int orc_moments(const orc_op* o, const double* ql, const double* qr, double out[4]) {
  double r[4] = {0, 0, 0, 0}, dn = 0.0;
  const int L = o->L;
  if (o->kind == O_Y2AT) { /* TMat/tmat.cpp:309-314: not implemented there */
    for (int k = 0; k < 4; ++k) out[k] = 0.0;
    return -1;
  }
  const st_t lmask = (1ull << L) - 1;
  for (int64_t i = 0; i < o->n; ++i) {
    st_t s = o->tab.n ? o->tab.idx[i] : (st_t)i;
    /* two-layer states: GenMatPhys::moments takes the low layer
     * (TMat/tmatphys.cpp:71-98), YAMMatVecProd2D::moments the left (high)
     * layer of the representative (TMat/tmatreduce.cpp:878-905) */
    if (o->kind == O_YAT) s &= lmask;
    if (o->kind == O_YAM) s >>= L;
    double w = o->sym ? ql[i] * ql[i] : ql[i] * qr[i];
    double p = bzexp1(s, L), m = p;
    dn += w;
    for (int k = 0; k < 4; ++k) {
      r[k] += m * w;
      m *= p;
    }
  }
  for (int k = 0; k < 4; ++k) out[k] = o->sym ? r[k] / L : r[k] / (L * dn);
  return o->kind == O_ZBM ? -1 : 0;
}

/* phys_extend: TMat/tmatphys.cpp:40-59, 100-106; TMat/tmatreduce.cpp:593-613,
 * 1289-1320, 1777-1781; TMat/tmat3d.cpp:165-177 */
int orc_phys_extend(const orc_op* o, const double* ql, const double* qr, double* out, int cap, int* nout) {
  const int L = o->L;
  *nout = 0;
  if (o->kind == O_XAT || o->kind == O_XAM || o->kind == O_XDT) {
    double a = 0, b = 0;
    int bc = (o->kind == O_XDT) ? 0 : o->mphys_bc;
    for (int64_t i = 0; i < o->n; ++i) {
      st_t s = o->tab.n ? o->tab.idx[i] : (st_t)i;
      double m = nnode(s, L, bc), w = ql[i] * ql[i];
      a += m * w;
      b += m * m * w;
    }
    if (cap >= 2) {
      out[0] = a;
      out[1] = b;
    }
    *nout = 2;
    return 0;
  }
  if (o->kind == O_XDM) {
    const st_t mask = o->nstate - 1, sf = 0xaaaaaaaaaaaaaaaaull;
    double r[4] = {0, 0, 0, 0};
    for (int64_t i = 0; i < o->n; ++i) {
      st_t s = o->tab.idx[i];
      double dm = bzexp1((s ^ sf) & mask, L), dmb = bzexp1(s, L), w = ql[i] * ql[i];
      r[0] += fabs(dm) * w;
      r[1] += fabs(dmb) * w;
      r[2] += dm * dm * w;
      r[3] += dmb * dmb * w;
    }
    r[0] /= L;
    r[1] /= L;
    r[2] /= L * L;
    r[3] /= L * L;
    for (int k = 0; k < 4 && k < cap; ++k) out[k] = r[k];
    *nout = 4;
    return 0;
  }
  if (o->kind == O_X3D) {
    if (cap >= 2) out[0] = out[1] = NAN;
    *nout = 2;
    return -1;
  }
  if (o->kind == O_ZBM) return -1;
  return 0;
}
