/*
 * imsrg_oracle.c -- CPU oracle for the IMSRG(2) scalar commutator engine.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker that the GPU library is
 * compared against; it is never linked into, called by, or shipped with the
 * product library.  Only tests/, __graft_entry__.smoke() and the CPU-baseline
 * leg of bench.py load it.
 *
 * It is a plain-C restatement of the reference Fortran routines on the hot
 * path of n-parzuchowski/EOM-IMSRG_FULL (paths relative to im-SRG/):
 *   basis + block layout      basic_IMSRG.f90:217-400, 477-641
 *   element access            basic_IMSRG.f90:1136-1177, 1270-1385, 2007-2046
 *   6j symbols                anglib.f:263-377 (d6ji), basic_IMSRG.f90:2509-2555
 *   operator arithmetic       basic_IMSRG.f90:2942-2969, 3450-3562, 3921-3952
 *   mbpt2, normal_order       basic_IMSRG.f90:4030-4064, 2375-2506
 *   vectorize / repackage     basic_IMSRG.f90:3794-3918
 *   cross-coupled layout      cross_coupled.f90:61-177, 1167-1300, 2196-2210
 *   commutators               commutators.f90:10-925
 *   White generator           generators.f90:4-106
 *   Magnus / BCH / Euler      IMSRG_MAGNUS.f90:15-234, 622-693, 756-766
 *   brute-force checks        brute_force_testing.f90:1765-1823, 1887-1928,
 *                             1975-2076; anglib.f:531-566 (wcoeff, coef9)
 *
 * The reference cannot be compiled here (no Fortran compiler), so parity of
 * this restatement is pinned by the reference's own known-answer test: the
 * brute-force uncoupled/9j formulas of brute_force_testing.f90, restated at
 * the bottom of this file and exercised by tests/test_oracle_pin.py with the
 * reference's tolerances (1e-10 zero/one-body, 1e-6 two-body).
 *
 * Conventions kept from the reference: orbit indices are 1-based, all angular
 * momenta are doubled (jj = 2j, J2 = 2J, itzp = 2tz), matrices are Fortran
 * column-major.  The Fortran COMMON-block cache behind v_same
 * (basic_IMSRG.f90:1282, 2015) becomes an explicit location record.
 *
 * Operator storage ("flat layout", shared by oracle, tests and the GPU library):
 *   [0]            E0
 *   fhh  A x A     column-major
 *   fph  P x A
 *   fpp  P x P
 *   for q = 1..nblocks, g = 1..6: gam(g) of block q, n1 x n2 column-major,
 *     g = 1 pppp (npp,npp), 2 ppph (npp,nph), 3 pphh (npp,nhh),
 *         4 phph (nph,nph), 5 hhhh (nhh,nhh), 6 phhh (nph,nhh)
 *     (basic_IMSRG.f90:579-584).
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORC_MAXJ 64

/* public tables of basic_IMSRG.f90:120-133 */
static const int sea1[6] = {1, 1, 1, 2, 3, 2};
static const int sea2[6] = {1, 2, 3, 2, 3, 3};
static const int sqs[6] = {1, 0, 0, 1, 1, 0};
static const int jst[6] = {10000000, 1, 1, 10000000, 10000000, 1};

typedef struct {
  int n1, n2;
  long off;
} ogam;

typedef struct {
  int J2, par, tz;
  int npp, nph, nhh;
  int *qn[3]; /* qn[c][2*(IX-1)+k], k=0,1 : orbit (1-based) */
  ogam gam[6];
} oblock;

typedef struct {
  int norb, A, P;
  int *nn, *ll, *jj, *itzp, *con; /* 1-based */
  int *holes, *parts;             /* 1-based lists */
  int *hb4, *pb4;
  int Jtotal_max, lmax;
  int nblocks;
  oblock *blk;
  int *xmap_jmin;
  int **xmap;
  int spblocks;
  int **states;
  int *nstates;
  long nfull, neq;
  long off_fhh, off_fph, off_fpp;
  /* cross-coupled layout (cross_coupled.f90:61-177) */
  int ccblocks;
  int *cc_nph, *cc_rlen, *cc_J2;
  int *cc_row; /* [q1-1][i-1][j-1] -> row (1-based) or 0 */
  int *cc_col; /* [q1-1][i-1][j-1] -> nb col (1-based) or 0 */
  long *cc_off, cc_total;
  long *wcc_off, wcc_total;
  /* 6j cache: [j1h][j2h][j4h][j5h][J3][J6] */
  int nj, nJ;
  double *six;
  double dfactl[1001];
} obasis;

typedef struct {
  int C1, C2, q, qx, i1, i2;
  double pre;
  int fail;
} vloc;

/* ------------------------------------------------------------------ */
/* small helpers                                                       */
/* ------------------------------------------------------------------ */
static int iabs_(int x) { return x < 0 ? -x : x; }
static int imax_(int a, int b) { return a > b ? a : b; }
static int imin_(int a, int b) { return a < b ? a : b; }
static int imod_(int a, int n) { return a % n; } /* Fortran mod, a >= 0 here */
static double ipow_m1(int e) { return (e % 2 == 0) ? 1.0 : -1.0; } /* (-1)**e, e may be < 0 */

/* basic_IMSRG.f90:1049-1061 */
static int triangle(int j1, int j2, int J) { return (J <= j1 + j2) && (J >= iabs_(j1 - j2)); }
/* basic_IMSRG.f90:1064-1070 */
static int block_index(int J, int T, int P) { return 3 * J + 2 * (T + 1) + P + 1; }
/* basic_IMSRG.f90:3576-3585 */
static int bosonic_tp_index(int i, int j, int n) { return n * (i - 1) + (3 * i - i * i) / 2 + j - i; }

/* ------------------------------------------------------------------ */
/* 6j symbols: anglib.f:263-377                                         */
/* ------------------------------------------------------------------ */
static void dfact0(obasis *b) {
  b->dfactl[0] = 0.0;
  for (int i = 1; i <= 1000; i++) b->dfactl[i] = b->dfactl[i - 1] + log((double)i);
}

static double dtri(const obasis *b, int j, int k, int l) {
  double d = b->dfactl[(j + k - l) / 2] + b->dfactl[(j - k + l) / 2] + b->dfactl[(-j + k + l) / 2] -
             b->dfactl[(j + k + l) / 2 + 1];
  return d * 0.5;
}

static double wwwwww(const obasis *b, double df, int j1, int j2, int j3, int l1, int l2, int l3) {
  int m1 = (j1 + j2 + j3) / 2, m2 = (j1 + l2 + l3) / 2, m3 = (l1 + j2 + l3) / 2, m4 = (l1 + l2 + j3) / 2;
  int m5 = (j1 + j2 + l1 + l2) / 2, m6 = (j2 + j3 + l2 + l3) / 2, m7 = (j3 + j1 + l3 + l1) / 2;
  int imin = imax_(imax_(m1, m2), imax_(m3, m4));
  int imax = imin_(imin_(m5, m6), m7);
  double w0 = 0.0;
  for (int i = imin; i <= imax; i++) {
    double sign = (i & 1) ? -1.0 : 1.0;
    w0 += sign * exp(df + b->dfactl[i + 1] - b->dfactl[i - m1] - b->dfactl[i - m2] - b->dfactl[i - m3] -
                     b->dfactl[i - m4] - b->dfactl[m5 - i] - b->dfactl[m6 - i] - b->dfactl[m7 - i]);
  }
  return w0;
}

static double d6ji(const obasis *b, int j1, int j2, int j3, int l1, int l2, int l3) {
  if (j1 < 0 || j2 < 0 || j3 < 0 || l1 < 0 || l2 < 0 || l3 < 0) return 0.0;
  if (j1 < iabs_(j2 - j3) || j1 > j2 + j3 || j3 < iabs_(l1 - l2) || j3 > l1 + l2 || j2 < iabs_(l1 - l3) ||
      j2 > l1 + l3 || j1 < iabs_(l2 - l3) || j1 > l2 + l3)
    return 0.0;
  if (((j1 + j2 + j3) & 1) || ((j3 + l1 + l2) & 1) || ((j2 + l1 + l3) & 1) || ((j1 + l2 + l3) & 1)) return 0.0;
  double df = dtri(b, j1, j2, j3) + dtri(b, j1, l2, l3) + dtri(b, l1, j2, l3) + dtri(b, l1, l2, j3);
  return wwwwww(b, df, j1, j2, j3, l1, l2, l3);
}

/* basic_IMSRG.f90:2509-2555: triangle check, then the stored value, which
 * store_6j computed with (j1,j2) ordered and (j4,j5) swapped alongside. */
static double sixj_raw(const obasis *b, int j1, int j2, int j3, int j4, int j5, int j6) {
  if (!(triangle(j1, j2, j3) && triangle(j4, j5, j3) && triangle(j1, j5, j6) && triangle(j4, j2, j6))) return 0.0;
  int l1 = j1, l2 = j2, l4 = j4, l5 = j5;
  if (j1 > j2) {
    l1 = j2; l2 = j1; l4 = j5; l5 = j4;
  }
  return d6ji(b, l1, l2, j3, l4, l5, j6);
}

static void build_sixj_cache(obasis *b) {
  b->nj = (b->Jtotal_max + 1) / 2;       /* single-particle 2j = 1,3,..,Jtotal_max */
  b->nJ = b->Jtotal_max + 1;             /* pair 2J = 0,2,..,2*Jtotal_max */
  long n = (long)b->nj * b->nj * b->nj * b->nj * b->nJ * b->nJ;
  b->six = (double *)calloc(n, sizeof(double));
  for (int a = 0; a < b->nj; a++)
    for (int c = 0; c < b->nj; c++)
      for (int d = 0; d < b->nj; d++)
        for (int e = 0; e < b->nj; e++)
          for (int J3 = 0; J3 < b->nJ; J3++)
            for (int J6 = 0; J6 < b->nJ; J6++) {
              long idx = ((((long)a * b->nj + c) * b->nj + d) * b->nj + e) * b->nJ * b->nJ + J3 * b->nJ + J6;
              b->six[idx] = sixj_raw(b, 2 * a + 1, 2 * c + 1, 2 * J3, 2 * d + 1, 2 * e + 1, 2 * J6);
            }
}

/* sixj(j1,j2,j3,j4,j5,j6): j1,j2,j4,j5 half-integer (doubled), j3,j6 integer (doubled) */
static double sixj(const obasis *b, int j1, int j2, int j3, int j4, int j5, int j6) {
  if (j3 < 0 || j6 < 0 || j3 / 2 >= b->nJ || j6 / 2 >= b->nJ || j1 > b->Jtotal_max || j2 > b->Jtotal_max ||
      j4 > b->Jtotal_max || j5 > b->Jtotal_max)
    return sixj_raw(b, j1, j2, j3, j4, j5, j6);
  long idx = (((((long)(j1 - 1) / 2) * b->nj + (j2 - 1) / 2) * b->nj + (j4 - 1) / 2) * b->nj + (j5 - 1) / 2) *
                 b->nJ * b->nJ +
             (j3 / 2) * b->nJ + j6 / 2;
  return b->six[idx];
}

/* anglib.f:531-541 */
static double wcoeff(const obasis *b, int ia, int ib, int ic, int id, int ie, int iff) {
  double w = d6ji(b, ia, ib, ie, id, ic, iff);
  if ((((ia + ib + ic + id) / 2) & 1) == 1) w = -w;
  return w;
}

/* anglib.f:546-566 */
static double coef9(const obasis *b, int j1, int j2, int j3, int j4, int j5, int j6, int j7, int j8, int j9) {
  double c = 0.0;
  int kmin = imax_(imax_(iabs_(j1 - j9), iabs_(j4 - j8)), iabs_(j2 - j6));
  int kmax = imin_(imin_(j1 + j9, j4 + j8), j2 + j6);
  if (kmin > kmax) return 0.0;
  for (int k = kmin; k <= kmax; k += 2)
    c += (k + 1) * wcoeff(b, j1, j9, j4, j8, k, j7) * wcoeff(b, j2, j6, j8, j4, k, j5) *
         wcoeff(b, j1, j9, j2, j6, k, j3);
  return c;
}

/* ------------------------------------------------------------------ */
/* basis construction                                                  */
/* ------------------------------------------------------------------ */
#define GAM(b, op, q, g) ((op) + (b)->blk[(q)-1].gam[(g)-1].off)
#define GX(b, op, q, g, i, j) \
  ((op)[(b)->blk[(q)-1].gam[(g)-1].off + ((long)(i)-1) + ((long)(j)-1) * (b)->blk[(q)-1].gam[(g)-1].n1])
#define QN(b, q, c, IX, k) ((b)->blk[(q)-1].qn[(c)-1][2 * ((IX)-1) + (k)-1])
#define FHH(b, op, i, j) ((op)[(b)->off_fhh + ((i)-1) + (long)((j)-1) * (b)->A])
#define FPH(b, op, i, j) ((op)[(b)->off_fph + ((i)-1) + (long)((j)-1) * (b)->P])
#define FPP(b, op, i, j) ((op)[(b)->off_fpp + ((i)-1) + (long)((j)-1) * (b)->P])

static void build_cc_layout(obasis *b);

obasis *orc_basis_new(int norb, const int *nn, const int *ll, const int *jj, const int *itzp, const int *con) {
  obasis *b = (obasis *)calloc(1, sizeof(obasis));
  b->norb = norb;
  int N = norb;
  b->nn = calloc(N + 1, sizeof(int));
  b->ll = calloc(N + 1, sizeof(int));
  b->jj = calloc(N + 1, sizeof(int));
  b->itzp = calloc(N + 1, sizeof(int));
  b->con = calloc(N + 1, sizeof(int));
  b->hb4 = calloc(N + 1, sizeof(int));
  b->pb4 = calloc(N + 1, sizeof(int));
  for (int i = 1; i <= N; i++) {
    b->nn[i] = nn[i - 1];
    b->ll[i] = ll[i - 1];
    b->jj[i] = jj[i - 1];
    b->itzp[i] = itzp[i - 1];
    b->con[i] = con[i - 1];
  }
  /* find_holes, basic_IMSRG.f90:380-398 */
  int A = 0;
  for (int i = 1; i <= N; i++) A += b->con[i];
  b->A = A;
  b->P = N - A;
  b->holes = calloc(A + 1, sizeof(int));
  b->parts = calloc(N - A + 1, sizeof(int));
  int r1 = 1, r2 = 1, hsum = 0;
  for (int i = 1; i <= N; i++) {
    b->hb4[i] = hsum;
    b->pb4[i] = i - b->hb4[i] - 1;
    if (b->con[i] == 1) b->holes[r1++] = i;
    else b->parts[r2++] = i;
    hsum += b->con[i];
  }
  b->Jtotal_max = 0;
  b->lmax = 0;
  for (int i = 1; i <= N; i++) {
    if (b->jj[i] > b->Jtotal_max) b->Jtotal_max = b->jj[i];
    if (b->ll[i] > b->lmax) b->lmax = b->ll[i];
  }
  dfact0(b);
  build_sixj_cache(b);

  /* jbas%states, basic_IMSRG.f90:302-340 */
  b->spblocks = (b->Jtotal_max + 1) * (b->lmax + 1);
  b->states = calloc(b->spblocks + 1, sizeof(int *));
  b->nstates = calloc(b->spblocks + 1, sizeof(int));
  int q = 1;
  for (int tzi = -1; tzi <= 1; tzi += 2)
    for (int li = 0; li <= b->lmax; li++)
      for (int ji = 1; ji <= b->Jtotal_max; ji += 2) {
        int r = 0;
        for (int i = 1; i <= N; i++)
          if (b->jj[i] == ji && b->ll[i] == li && b->itzp[i] == tzi) r++;
        b->states[q] = calloc(r + 1, sizeof(int));
        b->nstates[q] = r;
        r = 0;
        for (int i = 1; i <= N; i++)
          if (b->jj[i] == ji && b->ll[i] == li && b->itzp[i] == tzi) b->states[q][++r] = i;
        q++;
      }

  /* allocate_blocks, basic_IMSRG.f90:477-641 */
  b->nblocks = (b->Jtotal_max + 1) * 6;
  b->blk = calloc(b->nblocks + 1, sizeof(oblock));
  int nx = N * (N + 1) / 2;
  b->xmap = calloc(nx + 1, sizeof(int *));
  b->xmap_jmin = calloc(nx + 1, sizeof(int));
  for (int i = 1; i <= N; i++)
    for (int j = i; j <= N; j++) {
      int jmin = iabs_(b->jj[i] - b->jj[j]);
      int jmax = b->jj[i] + b->jj[j];
      int numJ = (jmax - jmin) / 2 + 2;
      int x = bosonic_tp_index(i, j, N);
      b->xmap[x] = calloc(numJ + 1, sizeof(int));
      b->xmap_jmin[x] = jmin;
    }
  b->off_fhh = 1;
  b->off_fph = b->off_fhh + (long)A * A;
  b->off_fpp = b->off_fph + (long)(N - A) * A;
  long off = b->off_fpp + (long)(N - A) * (N - A);
  long neq = 1 + (long)A * A + (long)(N - A) * (N - A) + (long)(N - A) * A;
  q = 1;
  for (int Jtot = 0; Jtot <= 2 * b->Jtotal_max; Jtot += 2)
    for (int Tz = -1; Tz <= 1; Tz++)
      for (int Par = 0; Par <= 1; Par++) {
        oblock *B = &b->blk[q - 1];
        B->J2 = Jtot;
        B->par = Par;
        B->tz = Tz;
        int np = 0, nb = 0, nh = 0;
        for (int pass = 0; pass < 2; pass++) {
          np = nb = nh = 0;
          for (int i = 1; i <= N; i++)
            for (int j = i; j <= N; j++) {
              if (Tz != (b->itzp[i] + b->itzp[j]) / 2) continue;
              if (Par != (1 - (int)ipow_m1(b->ll[i] + b->ll[j])) / 2) continue;
              if (!triangle(b->jj[i], b->jj[j], Jtot)) continue;
              int CX = b->con[i] + b->con[j];
              int x = bosonic_tp_index(i, j, N);
              int jmin = b->xmap_jmin[x];
              int c = CX + 1; /* qn(1)=pp, qn(2)=ph, qn(3)=hh */
              int *cnt = (CX == 0) ? &np : (CX == 1) ? &nb : &nh;
              (*cnt)++;
              if (pass == 1) {
                B->qn[c - 1][2 * (*cnt - 1)] = i;
                B->qn[c - 1][2 * (*cnt - 1) + 1] = j;
                b->xmap[x][(Jtot - jmin) / 2 + 1] = *cnt; /* Z((Jtot-jmin)/2+2), Z(1)=jmin */
              }
            }
          if (pass == 0) {
            B->npp = np;
            B->nph = nb;
            B->nhh = nh;
            B->qn[0] = calloc(2 * np + 2, sizeof(int));
            B->qn[1] = calloc(2 * nb + 2, sizeof(int));
            B->qn[2] = calloc(2 * nh + 2, sizeof(int));
          }
        }
        int d1[6] = {np, np, np, nb, nh, nb};
        int d2[6] = {np, nb, nh, nb, nh, nh};
        for (int g = 0; g < 6; g++) {
          B->gam[g].n1 = d1[g];
          B->gam[g].n2 = d2[g];
          B->gam[g].off = off;
          off += (long)d1[g] * d2[g];
          if (sqs[g]) neq += (long)d1[g] * (d1[g] + 1) / 2;
          else neq += (long)d1[g] * d2[g];
        }
        q++;
      }
  b->nfull = off;
  b->neq = neq;
  build_cc_layout(b);
  return b;
}

/* allocate_CCMAT, cross_coupled.f90:61-177: rows are all ordered pairs (i,j)
 * allowed in the block, columns the (particle, hole) pairs among them. The
 * qmap/rmap/nbmap search of fetch_rval becomes a dense (block, i, j) table. */
static void build_cc_layout(obasis *b) {
  int N = b->norb, JTM = b->Jtotal_max;
  b->ccblocks = (JTM + 1) * 2 * 2;
  b->cc_nph = calloc(b->ccblocks + 1, sizeof(int));
  b->cc_rlen = calloc(b->ccblocks + 1, sizeof(int));
  b->cc_J2 = calloc(b->ccblocks + 1, sizeof(int));
  b->cc_row = calloc((long)b->ccblocks * N * N, sizeof(int));
  b->cc_col = calloc((long)b->ccblocks * N * N, sizeof(int));
  b->cc_off = calloc(b->ccblocks + 1, sizeof(long));
  b->wcc_off = calloc(b->ccblocks + 1, sizeof(long));
  long off = 0, woff = 0;
  for (int q1 = 1; q1 <= b->ccblocks; q1++) {
    int JC = imod_(q1 - 1, JTM + 1) * 2;
    int PAR = (q1 - 1) / (2 * JTM + 2);
    int TZ = imod_(q1 - 1, 2 * JTM + 2) / (JTM + 1);
    int nb = 0, r = 0;
    for (int i = 1; i <= N; i++)
      for (int j = 1; j <= N; j++) {
        if (!triangle(b->jj[i], b->jj[j], JC)) continue;
        if (imod_(b->ll[i] + b->ll[j], 2) != PAR) continue;
        if (iabs_(b->itzp[i] - b->itzp[j]) / 2 != TZ) continue;
        long x = ((long)(q1 - 1) * N + (i - 1)) * N + (j - 1);
        if (b->con[i] == 0 && b->con[j] == 1) b->cc_col[x] = ++nb;
        b->cc_row[x] = ++r;
      }
    b->cc_nph[q1] = nb;
    b->cc_rlen[q1] = r;
    b->cc_J2[q1] = JC;
    b->cc_off[q1 - 1] = off;
    b->wcc_off[q1 - 1] = woff;
    off += (long)r * nb;
    woff += (long)r * r;
  }
  b->cc_total = off;
  b->wcc_total = woff;
}

static int cc_rval(const obasis *b, int i, int j, int q1) {
  return b->cc_row[((long)(q1 - 1) * b->norb + (i - 1)) * b->norb + (j - 1)];
}
static int cc_nbval(const obasis *b, int i, int j, int q1) {
  return b->cc_col[((long)(q1 - 1) * b->norb + (i - 1)) * b->norb + (j - 1)];
}

void orc_basis_free(obasis *b) {
  if (!b) return;
  for (int q = 0; q < b->nblocks; q++)
    for (int c = 0; c < 3; c++) free(b->blk[q].qn[c]);
  free(b->blk);
  int nx = b->norb * (b->norb + 1) / 2;
  for (int x = 1; x <= nx; x++) free(b->xmap[x]);
  free(b->xmap);
  free(b->xmap_jmin);
  for (int q = 1; q <= b->spblocks; q++) free(b->states[q]);
  free(b->states);
  free(b->nstates);
  free(b->nn); free(b->ll); free(b->jj); free(b->itzp); free(b->con);
  free(b->holes); free(b->parts); free(b->hb4); free(b->pb4);
  free(b->cc_nph); free(b->cc_rlen); free(b->cc_J2); free(b->cc_row); free(b->cc_col);
  free(b->cc_off); free(b->wcc_off); free(b->six);
  free(b);
}

/* ------------------------------------------------------------------ */
/* element access                                                      */
/* ------------------------------------------------------------------ */
/* basic_IMSRG.f90:1136-1144 */
static int sp_block_index(const obasis *b, int j, int l, int t) {
  return ((t + 1) * (b->Jtotal_max + 1) * (b->lmax + 1)) / 4 + l * (b->Jtotal_max + 1) / 2 + (j + 1) / 2;
}

/* basic_IMSRG.f90:1147-1177 */
static double f_elem(const obasis *b, int a, int bb, const double *op, int herm) {
  int c1 = b->con[a], c2 = b->con[bb];
  switch (c1 + c2) {
    case 0: return FPP(b, op, a - b->hb4[a], bb - b->hb4[bb]);
    case 1:
      if (c1 > c2) return FPH(b, op, bb - b->hb4[bb], a - b->pb4[a]) * herm;
      return FPH(b, op, a - b->hb4[a], bb - b->pb4[bb]);
    default: return FHH(b, op, a - b->pb4[a], bb - b->pb4[bb]);
  }
}

static int xmap_row(const obasis *b, int i, int j, int J) {
  int x = bosonic_tp_index(i, j, b->norb);
  int jmin = b->xmap_jmin[x];
  return b->xmap[x][(J - jmin) / 2 + 1];
}

/* basic_IMSRG.f90:1270-1385 (pphh_ph is .false. for every operator on this
 * path). The location of a found element is returned for v_same. */
static double v_elem_loc(const obasis *b, int a, int bb, int c, int d, int J, const double *op, int herm,
                         vloc *loc) {
  vloc dummy;
  if (!loc) loc = &dummy;
  loc->fail = 1;
  int ja = b->jj[a], jb = b->jj[bb], jc = b->jj[c], jd = b->jj[d];
  if (!(triangle(ja, jb, J) && triangle(jc, jd, J))) return 0.0;
  int P = imod_(b->ll[a] + b->ll[bb], 2);
  if (imod_(b->ll[c] + b->ll[d], 2) != P) return 0.0;
  int T = (b->itzp[a] + b->itzp[bb]) / 2;
  if (b->itzp[c] + b->itzp[d] != 2 * T) return 0.0;
  int q = block_index(J, T, P);
  int C1 = b->con[a] + b->con[bb] + 1;
  int C2 = b->con[c] + b->con[d] + 1;
  int qx = C1 * C2;
  if (qx == 9) qx = 5; /* adjust_index(9) = -4 */
  double pre = 1.0;
  int i1, i2;
  if (a > bb) {
    i1 = xmap_row(b, bb, a, J);
    pre = ipow_m1(1 + (ja + jb - J) / 2);
  } else {
    if (a == bb) pre = pre * sqrt(2.0);
    i1 = xmap_row(b, a, bb, J);
  }
  if (c > d) {
    i2 = xmap_row(b, d, c, J);
    pre = pre * ipow_m1(1 + (jc + jd - J) / 2);
  } else {
    if (c == d) pre = pre * sqrt(2.0);
    i2 = xmap_row(b, c, d, J);
  }
  double v;
  if (C1 > C2) v = GX(b, op, q, qx, i2, i1) * herm * pre;
  else v = GX(b, op, q, qx, i1, i2) * pre;
  loc->C1 = C1; loc->C2 = C2; loc->q = q; loc->qx = qx; loc->i1 = i1; loc->i2 = i2; loc->pre = pre;
  loc->fail = 0;
  return v;
}

static double v_elem(const obasis *b, int a, int bb, int c, int d, int J, const double *op, int herm) {
  return v_elem_loc(b, a, bb, c, d, J, op, herm, NULL);
}

/* basic_IMSRG.f90:2007-2028 */
static double v_same(const obasis *b, const double *op, int herm, const vloc *loc) {
  if (loc->fail) return 0.0;
  if (loc->C1 > loc->C2) return GX(b, op, loc->q, loc->qx, loc->i2, loc->i1) * herm * loc->pre;
  return GX(b, op, loc->q, loc->qx, loc->i1, loc->i2) * loc->pre;
}

/* basic_IMSRG.f90:2031-2046 */
static double twobody_monopole(const obasis *b, int a, int bb, int ja, int jb, const double *H, int herm) {
  double sm = 0.0;
  for (int JT = iabs_(ja - jb); JT <= ja + jb; JT += 2) sm += (JT + 1) * v_elem(b, a, bb, a, bb, JT, H, herm);
  return sm / (ja + 1.0) / (jb + 1.0);
}

/* ------------------------------------------------------------------ */
/* dense FP64 GEMM with BLAS dgemm semantics (column-major)            */
/* ------------------------------------------------------------------ */
/* op(A) and op(B) are packed column-major, then each 8-column x 128-row tile
 * of C is accumulated as rank-1 updates over k (the i loop vectorises without
 * reassociation). */
#define GEMM_NB 8
#define GEMM_MB 128
/* An external BLAS dgemm (Fortran interface with 64-bit integers, e.g. the
 * OpenBLAS that numpy bundles) used in place of the oracle's own GEMM when set
 * by orc_set_dgemm: the timed CPU baseline, where the reference links a system
 * BLAS (makefile_gfortran:14).  Calls whose arguments a BLAS would reject
 * (empty contraction, leading dimension 0) stay with the oracle's own GEMM. */
typedef void (*ext_dgemm_t)(const char *, const char *, const long *, const long *, const long *, const double *,
                            const double *, const long *, const double *, const long *, const double *, double *,
                            const long *, size_t, size_t);
static ext_dgemm_t g_ext_dgemm = 0;
void orc_set_dgemm(void *fn) { g_ext_dgemm = (ext_dgemm_t)fn; }

static void dgemm_(char ta, char tb, int m, int n, int k, double alpha, const double *A, int lda, const double *B,
                   int ldb, double beta, double *C, int ldc) {
  if (m <= 0 || n <= 0) return;
  if (g_ext_dgemm && k > 0 && lda >= ((ta == 'N') ? m : k) && ldb >= ((tb == 'N') ? k : n) && ldc >= m) {
    const long M = m, N = n, K = k, LDA = lda, LDB = ldb, LDC = ldc;
    g_ext_dgemm(&ta, &tb, &M, &N, &K, &alpha, A, &LDA, B, &LDB, &beta, C, &LDC, 1, 1);
    return;
  }
  double *Ap = malloc(((long)m * (k > 0 ? k : 1)) * sizeof(double));
  double *Bp = malloc(((long)k * n + 1) * sizeof(double));
  for (int l = 0; l < k; l++)
    for (int i = 0; i < m; i++) Ap[i + (long)l * m] = (ta == 'N') ? A[i + (long)l * lda] : A[l + (long)i * lda];
  for (int j = 0; j < n; j++)
    for (int l = 0; l < k; l++) Bp[l + (long)j * k] = (tb == 'N') ? B[l + (long)j * ldb] : B[j + (long)l * ldb];
  int nj = (n + GEMM_NB - 1) / GEMM_NB, ni = (m + GEMM_MB - 1) / GEMM_MB;
  long work = (long)m * n * (k > 0 ? k : 1);
#pragma omp parallel for schedule(dynamic) collapse(2) if (work > 200000)
  for (int jb = 0; jb < nj; jb++)
    for (int ib = 0; ib < ni; ib++) {
      double acc[GEMM_NB][GEMM_MB];
      int j0 = jb * GEMM_NB, i0 = ib * GEMM_MB;
      int jn = (n - j0 < GEMM_NB) ? n - j0 : GEMM_NB;
      int in = (m - i0 < GEMM_MB) ? m - i0 : GEMM_MB;
      for (int jj = 0; jj < GEMM_NB; jj++)
        for (int i = 0; i < GEMM_MB; i++) acc[jj][i] = 0.0;
      for (int l = 0; l < k; l++) {
        const double *a = Ap + i0 + (long)l * m;
        for (int jj = 0; jj < jn; jj++) {
          double bv = Bp[l + (long)(j0 + jj) * k];
          double *c = acc[jj];
          for (int i = 0; i < in; i++) c[i] += a[i] * bv;
        }
      }
      for (int jj = 0; jj < jn; jj++)
        for (int i = 0; i < in; i++) {
          long ci = (i0 + i) + (long)(j0 + jj) * ldc;
          double cv = (beta == 0.0) ? 0.0 : beta * C[ci];
          C[ci] = alpha * acc[jj][i] + cv;
        }
    }
  free(Ap);
  free(Bp);
}

/* ------------------------------------------------------------------ */
/* operator arithmetic                                                 */
/* ------------------------------------------------------------------ */
/* add_sq_op, basic_IMSRG.f90:3450-3478 */
void orc_add(const obasis *b, const double *A, double ax, const double *B, double bx, double *C) {
  for (long i = 0; i < b->nfull; i++) C[i] = A[i] * ax + B[i] * bx;
}

/* mat_frob_norm, basic_IMSRG.f90:3921-3952: fph and non-square gam count twice */
double orc_norm(const obasis *b, const double *op) {
  double s1 = 0, s2 = 0, s3 = 0;
  for (long i = 0; i < (long)b->A * b->A; i++) s1 += op[b->off_fhh + i] * op[b->off_fhh + i];
  for (long i = 0; i < (long)b->P * b->A; i++) s2 += op[b->off_fph + i] * op[b->off_fph + i];
  for (long i = 0; i < (long)b->P * b->P; i++) s3 += op[b->off_fpp + i] * op[b->off_fpp + i];
  double sm = s1 + 2 * s2 + s3;
  for (int q = 1; q <= b->nblocks; q++)
    for (int g = 1; g <= 6; g++) {
      const ogam *G = &b->blk[q - 1].gam[g - 1];
      double s = 0;
      for (long i = 0; i < (long)G->n1 * G->n2; i++) s += op[G->off + i] * op[G->off + i];
      sm += s;
      if (!sqs[g - 1]) sm += s;
    }
  return sqrt(sm);
}

/* mbpt2, basic_IMSRG.f90:4030-4064 */
double orc_mbpt2(const obasis *b, const double *H, int herm) {
  double sm = 0.0;
  for (int q = 1; q <= b->nblocks; q++) {
    const oblock *B = &b->blk[q - 1];
    double s1 = 0.0;
    for (int II = 1; II <= B->npp; II++) {
      int i = QN(b, q, 1, II, 1), j = QN(b, q, 1, II, 2);
      double fi = f_elem(b, i, i, H, herm), fj = f_elem(b, j, j, H, herm);
      for (int JJ = 1; JJ <= B->nhh; JJ++) {
        int k = QN(b, q, 3, JJ, 1), l = QN(b, q, 3, JJ, 2);
        double fk = f_elem(b, k, k, H, herm), fl = f_elem(b, l, l, H, herm);
        double eden = fk + fl - fi - fj;
        double x = GX(b, H, q, 3, II, JJ);
        s1 += x * x / eden;
      }
    }
    sm += (B->J2 + 1.0) * s1;
  }
  return sm;
}

/* ------------------------------------------------------------------ */
/* commutators, commutators.f90                                        */
/* ------------------------------------------------------------------ */
/* commutators.f90:10-33 */
double orc_comm110(const obasis *b, const double *L, int hL, const double *R, int hR) {
  double sm = 0.0;
  for (int i = 1; i <= b->A; i++) {
    int ji = b->jj[b->holes[i]];
    for (int a = 1; a <= b->P; a++)
      sm += (FPH(b, L, a, i) * FPH(b, R, a, i) * hL - FPH(b, R, a, i) * FPH(b, L, a, i) * hR) * (ji + 1);
  }
  return sm;
}

/* commutators.f90:399-432 */
double orc_comm220(const obasis *b, const double *L, int hL, const double *R, int hR) {
  if (hR * hL != -1) return 0.0;
  double sm = 0.0;
  for (int q = 1; q <= b->nblocks; q++) {
    const oblock *B = &b->blk[q - 1];
    double smx = 0.0;
    for (int IX = 1; IX <= B->npp; IX++)
      for (int JX = 1; JX <= B->nhh; JX++) smx -= GX(b, L, q, 3, IX, JX) * GX(b, R, q, 3, IX, JX) * hR;
    sm += smx * (B->J2 + 1);
  }
  return sm * 2.0;
}

/* commutators.f90:36-80 */
static void comm111(const obasis *b, const double *L, int hL, const double *R, int hR, double *RES) {
  int hol = b->A, par = b->P;
  double *th1 = calloc((long)hol * hol + 1, sizeof(double)), *th2 = calloc((long)hol * hol + 1, sizeof(double));
  double *tb1 = calloc((long)par * hol + 1, sizeof(double)), *tb2 = calloc((long)par * hol + 1, sizeof(double));
  double *tp1 = calloc((long)par * par + 1, sizeof(double)), *tp2 = calloc((long)par * par + 1, sizeof(double));
  const double *Lhh = L + b->off_fhh, *Lph = L + b->off_fph, *Lpp = L + b->off_fpp;
  const double *Rhh = R + b->off_fhh, *Rph = R + b->off_fph, *Rpp = R + b->off_fpp;
  dgemm_('N', 'N', hol, hol, hol, 1.0, Lhh, hol, Rhh, hol, 0.0, th1, hol);
  dgemm_('T', 'N', hol, hol, par, 1.0, Lph, par, Rph, par, 0.0, th2, hol);
  for (int i = 0; i < hol; i++)
    for (int j = 0; j < hol; j++)
      RES[b->off_fhh + i + (long)j * hol] =
          th1[i + j * hol] + th2[i + j * hol] * hL - (th1[j + i * hol] * hL + th2[j + i * hol]) * hR;
  dgemm_('N', 'N', par, hol, hol, 1.0, Lph, par, Rhh, hol, 0.0, tb1, par);
  dgemm_('N', 'N', par, hol, par, 1.0, Lpp, par, Rph, par, 0.0, tb2, par);
  for (long i = 0; i < (long)par * hol; i++) RES[b->off_fph + i] = tb1[i] + tb2[i];
  dgemm_('N', 'N', par, hol, hol, 1.0, Rph, par, Lhh, hol, 0.0, tb1, par);
  dgemm_('N', 'N', par, hol, par, 1.0, Rpp, par, Lph, par, 0.0, tb2, par);
  for (long i = 0; i < (long)par * hol; i++) RES[b->off_fph + i] = RES[b->off_fph + i] - tb1[i] - tb2[i];
  dgemm_('N', 'T', par, par, hol, 1.0, Lph, par, Rph, par, 0.0, tp1, par);
  dgemm_('N', 'N', par, par, par, 1.0, Lpp, par, Rpp, par, 0.0, tp2, par);
  for (int i = 0; i < par; i++)
    for (int j = 0; j < par; j++)
      RES[b->off_fpp + i + (long)j * par] =
          tp1[i + (long)j * par] * hR + tp2[i + (long)j * par] - (tp1[j + (long)i * par] + tp2[j + (long)i * par] * hR) * hL;
  free(th1); free(th2); free(tb1); free(tb2); free(tp1); free(tp2);
}

/* one inner (a,i) sum of commutator_121, commutators.f90:117-150 */
static double c121_inner(const obasis *b, int pk, int qk, const double *L, int hL, const double *R, int hR) {
  int jq = b->jj[qk];
  double sm = 0.0;
  for (int a = 1; a <= b->P; a++) {
    int ak = b->parts[a];
    int ja = b->jj[ak], ta = b->itzp[ak], la = b->ll[ak];
    for (int i = 1; i <= b->A; i++) {
      int ik = b->holes[i];
      int ji = b->jj[ik], ti = b->itzp[ik], li = b->ll[ik];
      if (ji != ja || li != la || ti != ta) continue;
      double smx = 0, smy = 0, smx2 = 0, smy2 = 0;
      vloc loc;
      for (int JT = iabs_(ji - jq); JT <= ji + jq; JT += 2) {
        smx += v_elem_loc(b, ak, pk, ik, qk, JT, R, hR, &loc) * (JT + 1);
        smx2 += v_same(b, L, hL, &loc) * (JT + 1);
        smy += v_elem_loc(b, ik, pk, ak, qk, JT, R, hR, &loc) * (JT + 1);
        smy2 += v_same(b, L, hL, &loc) * (JT + 1);
      }
      sm += FPH(b, L, a, i) * (hL * smx - smy) - FPH(b, R, a, i) * (hR * smx2 - smy2);
    }
  }
  return sm;
}

/* commutators.f90:83-280 */
static void comm121(const obasis *b, const double *L, int hL, const double *R, int hR, double *RES, int hRES) {
  for (int p = 1; p <= b->A; p++) {
    int pk = b->holes[p];
    for (int q = p; q <= b->A; q++) {
      int qk = b->holes[q];
      if (b->jj[qk] != b->jj[pk] || b->ll[qk] != b->ll[pk] || b->itzp[qk] != b->itzp[pk]) continue;
      double sm = c121_inner(b, pk, qk, L, hL, R, hR);
      FHH(b, RES, p, q) = FHH(b, RES, p, q) + sm / (b->jj[pk] + 1.0);
      FHH(b, RES, q, p) = FHH(b, RES, p, q) * hRES;
    }
  }
  for (int p = 1; p <= b->P; p++) {
    int pk = b->parts[p];
    for (int q = p; q <= b->P; q++) {
      int qk = b->parts[q];
      if (b->jj[qk] != b->jj[pk] || b->ll[qk] != b->ll[pk] || b->itzp[qk] != b->itzp[pk]) continue;
      double sm = c121_inner(b, pk, qk, L, hL, R, hR);
      FPP(b, RES, p, q) = FPP(b, RES, p, q) + sm / (b->jj[pk] + 1.0);
      FPP(b, RES, q, p) = FPP(b, RES, p, q) * hRES;
    }
  }
  for (int p = 1; p <= b->P; p++) {
    int pk = b->parts[p];
    for (int q = 1; q <= b->A; q++) {
      int qk = b->holes[q];
      if (b->jj[qk] != b->jj[pk] || b->ll[qk] != b->ll[pk] || b->itzp[qk] != b->itzp[pk]) continue;
      double sm = c121_inner(b, pk, qk, L, hL, R, hR);
      FPH(b, RES, p, q) = FPH(b, RES, p, q) + sm / (b->jj[pk] + 1.0);
    }
  }
}

/* commutators.f90:283-396 */
static void comm122(const obasis *b, const double *L, int hL, const double *R, int hR, double *RES, int hRES) {
#pragma omp parallel for schedule(dynamic)
  for (int q = 1; q <= b->nblocks; q++) {
    int JT = b->blk[q - 1].J2;
    for (int g = 1; g <= 6; g++) {
      int n1 = b->blk[q - 1].gam[g - 1].n1, n2 = b->blk[q - 1].gam[g - 1].n2;
      if (n1 * n2 == 0) continue;
      int c1 = sea1[g - 1], c2 = sea2[g - 1], square = sqs[g - 1], jxstart = jst[g - 1];
      for (int IX = 1; IX <= n1; IX++) {
        int a = QN(b, q, c1, IX, 1), bb = QN(b, q, c1, IX, 2);
        for (int JX = imin_(jxstart, IX); JX <= n2; JX++) {
          int c = QN(b, q, c2, JX, 1), d = QN(b, q, c2, JX, 2);
          double sm = 0.0;
          vloc loc;
          int qs = sp_block_index(b, b->jj[a], b->ll[a], b->itzp[a]);
          for (int i = 1; i <= b->nstates[qs]; i++) {
            int isp = b->states[qs][i];
            double vr = v_elem_loc(b, isp, bb, c, d, JT, R, hR, &loc);
            sm += f_elem(b, a, isp, L, hL) * vr - f_elem(b, a, isp, R, hR) * v_same(b, L, hL, &loc);
          }
          qs = sp_block_index(b, b->jj[bb], b->ll[bb], b->itzp[bb]);
          for (int i = 1; i <= b->nstates[qs]; i++) {
            int isp = b->states[qs][i];
            double vr = v_elem_loc(b, a, isp, c, d, JT, R, hR, &loc);
            sm += f_elem(b, bb, isp, L, hL) * vr - f_elem(b, bb, isp, R, hR) * v_same(b, L, hL, &loc);
          }
          qs = sp_block_index(b, b->jj[c], b->ll[c], b->itzp[c]);
          for (int i = 1; i <= b->nstates[qs]; i++) {
            int isp = b->states[qs][i];
            double vr = v_elem_loc(b, a, bb, isp, d, JT, R, hR, &loc);
            sm += -f_elem(b, isp, c, L, hL) * vr + f_elem(b, isp, c, R, hR) * v_same(b, L, hL, &loc);
          }
          qs = sp_block_index(b, b->jj[d], b->ll[d], b->itzp[d]);
          for (int i = 1; i <= b->nstates[qs]; i++) {
            int isp = b->states[qs][i];
            double vr = v_elem_loc(b, a, bb, c, isp, JT, R, hR, &loc);
            sm += -f_elem(b, isp, d, L, hL) * vr + f_elem(b, isp, d, R, hR) * v_same(b, L, hL, &loc);
          }
          sm = sm / sqrt(1.0 + (a == bb)) / sqrt(1.0 + (c == d));
          GX(b, RES, q, g, IX, JX) = sm;
          if (square) GX(b, RES, q, g, JX, IX) = sm * hRES;
        }
      }
    }
  }
}

/* commutators.f90:581-768.  w1, w2 are full operators (herm = +1). */
static void comm222_pphh(const obasis *b, const double *L, int hL, const double *R, int hR, double *RES,
                         double *w1, double *w2) {
  int pm = hR * hL;
  for (int q = 1; q <= b->nblocks; q++) {
    const oblock *B = &b->blk[q - 1];
    int nh = B->nhh, np = B->npp, nb = B->nph;
    for (int g = 1; g <= 6; g++) {
      long n = (long)B->gam[g - 1].n1 * B->gam[g - 1].n2;
      memset(GAM(b, w1, q, g), 0, n * sizeof(double));
      memset(GAM(b, w2, q, g), 0, n * sizeof(double));
    }
    const double *L1 = GAM(b, L, q, 1), *L2 = GAM(b, L, q, 2), *L3 = GAM(b, L, q, 3), *L5 = GAM(b, L, q, 5),
                 *L6 = GAM(b, L, q, 6);
    const double *R1 = GAM(b, R, q, 1), *R2 = GAM(b, R, q, 2), *R3 = GAM(b, R, q, 3), *R5 = GAM(b, R, q, 5),
                 *R6 = GAM(b, R, q, 6);
    double *W11 = GAM(b, w1, q, 1), *W12 = GAM(b, w1, q, 2), *W13 = GAM(b, w1, q, 3), *W14 = GAM(b, w1, q, 4),
           *W15 = GAM(b, w1, q, 5), *W16 = GAM(b, w1, q, 6);
    double *W21 = GAM(b, w2, q, 1), *W22 = GAM(b, w2, q, 2), *W23 = GAM(b, w2, q, 3), *W24 = GAM(b, w2, q, 4),
           *W25 = GAM(b, w2, q, 5), *W26 = GAM(b, w2, q, 6);
    if (np != 0) dgemm_('N', 'N', np, np, np, 1.0, L1, np, R1, np, 0.0, W11, np);
    if (nh != 0) dgemm_('N', 'N', nh, nh, nh, 1.0, L5, nh, R5, nh, 0.0, W25, nh);
    if (np * nh != 0) {
      dgemm_('T', 'N', nh, nh, np, 1.0, L3, np, R3, np, 0.0, W15, nh);
      for (long i = 0; i < (long)nh * nh; i++) W15[i] *= hL;
      dgemm_('N', 'T', np, np, nh, 1.0, L3, np, R3, np, 0.0, W21, np);
      for (long i = 0; i < (long)np * np; i++) W21[i] *= hR;
      dgemm_('N', 'N', np, nh, np, -1.0, R1, np, L3, np, 0.0, W13, np);
      dgemm_('N', 'N', np, nh, np, 1.0, L1, np, R3, np, 1.0, W13, np);
      dgemm_('N', 'N', np, nh, nh, 1.0, R3, np, L5, nh, 0.0, W23, np);
      dgemm_('N', 'N', np, nh, nh, 1.0, L3, np, R5, nh, -1.0, W23, np);
    }
    double *X1 = GAM(b, RES, q, 1), *X5 = GAM(b, RES, q, 5), *X3 = GAM(b, RES, q, 3);
    double *X4 = GAM(b, RES, q, 4), *X6 = GAM(b, RES, q, 6), *X2 = GAM(b, RES, q, 2);
    for (int i = 0; i < np; i++)
      for (int j = 0; j < np; j++) {
        long ij = i + (long)j * np, ji = j + (long)i * np;
        X1[ij] = X1[ij] + W11[ij] - W21[ij] - (W11[ji] - W21[ji]) * pm;
      }
    for (int i = 0; i < nh; i++)
      for (int j = 0; j < nh; j++) {
        long ij = i + (long)j * nh, ji = j + (long)i * nh;
        X5[ij] = X5[ij] + W15[ij] - W25[ij] - (W15[ji] - W25[ji]) * pm;
      }
    for (long i = 0; i < (long)np * nh; i++) X3[i] = X3[i] + W13[i] - W23[i];
    if (nb * nh != 0) {
      dgemm_('N', 'T', nb, nb, nh, 1.0, L6, nb, R6, nb, 0.0, W24, nb);
      for (long i = 0; i < (long)nb * nb; i++) W24[i] *= hR;
    }
    if (nb * np != 0) {
      dgemm_('T', 'N', nb, nb, np, 1.0, L2, np, R2, np, 0.0, W14, nb);
      for (long i = 0; i < (long)nb * nb; i++) W14[i] *= hL;
    }
    for (int i = 0; i < nb; i++)
      for (int j = 0; j < nb; j++) {
        long ij = i + (long)j * nb, ji = j + (long)i * nb;
        X4[ij] = X4[ij] + W14[ij] - W24[ij] - (W14[ji] - W24[ji]) * pm;
      }
    if (nb * nh != 0) {
      dgemm_('N', 'N', nb, nh, nh, 1.0, R6, nb, L5, nh, 0.0, W26, nb);
      dgemm_('N', 'N', nb, nh, nh, 1.0, L6, nb, R5, nh, -1.0, W26, nb);
    }
    if (nb * np != 0) {
      dgemm_('N', 'N', np, nb, np, 1.0, R1, np, L2, np, 0.0, W12, np);
      dgemm_('N', 'N', np, nb, np, 1.0, L1, np, R2, np, -1.0, W12, np);
    }
    if (nb * np * nh != 0) {
      dgemm_('T', 'N', nb, nh, np, -1.0 * hR, R2, np, L3, np, 0.0, W16, nb);
      dgemm_('T', 'N', nb, nh, np, (double)hL, L2, np, R3, np, 1.0, W16, nb);
      dgemm_('N', 'T', np, nb, nh, 1.0, R3, np, L6, nb, 0.0, W22, np);
      dgemm_('N', 'T', np, nb, nh, (double)hR, L3, np, R6, nb, -1.0 * hL, W22, np);
    }
    for (long i = 0; i < (long)nb * nh; i++) X6[i] = X6[i] + W16[i] - W26[i];
    for (long i = 0; i < (long)np * nb; i++) X2[i] = X2[i] + W12[i] - W22[i];
  }
}

/* commutators.f90:435-578 */
static void comm221(const obasis *b, int hL, int hR, double *RES, int hRES, const double *w1,
                    const double *w2) {
  int Abody = b->A, Ntot = b->norb;
  int pm = hR * hL;
  for (int pass = 0; pass < 3; pass++) {
    /* pass 0: fhh (i,j holes, j>=i); 1: fpp (j>=i); 2: fph (i part, j hole) */
    int ni = (pass == 0) ? Abody : Ntot - Abody;
    for (int i = 1; i <= ni; i++) {
      int ik = (pass == 0) ? b->holes[i] : b->parts[i];
      int ji = b->jj[ik], li = b->ll[ik], ti = b->itzp[ik];
      int jlo = (pass == 2) ? 1 : i;
      int jhi = (pass == 1) ? Ntot - Abody : Abody;
      for (int j = jlo; j <= jhi; j++) {
        int jk = (pass == 1) ? b->parts[j] : b->holes[j];
        if (b->jj[jk] != ji || b->ll[jk] != li || b->itzp[jk] != ti) continue;
        double sm = 0.0;
        for (int c = 1; c <= Abody; c++) {
          int ck = b->holes[c], jc = b->jj[ck];
          for (int JT = iabs_(jc - ji); JT <= jc + ji; JT += 2) {
            if (pass == 2) sm += v_elem(b, ck, ik, ck, jk, JT, w1, 1) * (JT + 1);
            else sm += (v_elem(b, ck, ik, ck, jk, JT, w1, 1) - pm * v_elem(b, ck, jk, ck, ik, JT, w1, 1)) * (JT + 1);
          }
        }
        for (int c = 1; c <= Ntot - Abody; c++) {
          int ck = b->parts[c], jc = b->jj[ck];
          for (int JT = iabs_(jc - ji); JT <= jc + ji; JT += 2) {
            if (pass == 2) sm += v_elem(b, ck, ik, ck, jk, JT, w2, 1) * (JT + 1);
            else sm += (v_elem(b, ck, ik, ck, jk, JT, w2, 1) - pm * v_elem(b, ck, jk, ck, ik, JT, w2, 1)) * (JT + 1);
          }
        }
        if (pass == 0) {
          FHH(b, RES, i, j) = FHH(b, RES, i, j) + sm / (ji + 1.0);
          FHH(b, RES, j, i) = FHH(b, RES, i, j) * hRES;
        } else if (pass == 1) {
          FPP(b, RES, i, j) = FPP(b, RES, i, j) + sm / (ji + 1.0);
          FPP(b, RES, j, i) = FPP(b, RES, i, j) * hRES;
        } else {
          FPH(b, RES, i, j) = FPH(b, RES, i, j) + sm / (ji + 1.0);
        }
      }
    }
  }
}

/* calculate_cross_coupled, cross_coupled.f90:1190-1300 */
void orc_cross_coupled(const obasis *b, const double *HS, int herm, double *CCX) {
  int Atot = b->A, Ntot = b->norb, JTM = b->Jtotal_max;
#pragma omp parallel for schedule(dynamic)
  for (int q1 = 1; q1 <= b->ccblocks; q1++) {
    int JC = imod_(q1 - 1, JTM + 1) * 2;
    int PAR = (q1 - 1) / (2 * JTM + 2);
    int TZ = imod_(q1 - 1, 2 * JTM + 2) / (JTM + 1);
    int rlen = b->cc_rlen[q1];
    double *X = CCX + b->cc_off[q1 - 1];
    memset(X, 0, (long)rlen * b->cc_nph[q1] * sizeof(double));
    for (int hg = 1; hg <= Atot; hg++)
      for (int pg = 1; pg <= Ntot - Atot; pg++) {
        int h = b->holes[hg], p = b->parts[pg];
        int jp = b->jj[p], jh = b->jj[h], lp = b->ll[p], lh = b->ll[h], tp = b->itzp[p], th = b->itzp[h];
        if (!triangle(jp, jh, JC)) continue;
        if (imod_(lp + lh, 2) != PAR) continue;
        if (iabs_(tp - th) / 2 != TZ) continue;
        int NBindx = cc_nbval(b, p, h, q1);
        for (int a = 1; a <= Ntot; a++)
          for (int bb = 1; bb <= Ntot; bb++) {
            int ja = b->jj[a], jb = b->jj[bb], la = b->ll[a], lb = b->ll[bb], ta = b->itzp[a], tb = b->itzp[bb];
            if (!triangle(ja, jb, JC)) continue;
            if (imod_(la + lb, 2) != PAR) continue;
            if (iabs_(ta - tb) / 2 != TZ) continue;
            int Rindx = cc_rval(b, a, bb, q1);
            if (imod_(la + lh, 2) == imod_(lb + lp, 2) && (ta + th) == (tb + tp)) {
              int Jmin = imax_(iabs_(jp - jb), iabs_(ja - jh));
              int Jmax = imin_(jp + jb, ja + jh);
              double sm = 0.0;
              for (int JT = Jmin; JT <= Jmax; JT += 2)
                sm += ipow_m1(JT / 2) * (JT + 1) * sixj(b, jp, jh, JC, ja, jb, JT) *
                      v_elem(b, h, a, p, bb, JT, HS, herm);
              X[(Rindx - 1) + (long)(NBindx - 1) * rlen] = sm * ipow_m1((jh + jb + JC) / 2) * 1.0 * sqrt(JC + 1.0);
            }
          }
      }
  }
}

/* commutators.f90:771-925 (the WCC GEMM of :792-802 included) */
static void comm222_ph(const obasis *b, const double *LCC, int hL, const double *RCC, int hR, double *RES,
                       int hRES, double *WCC) {
  int JTM = b->Jtotal_max;
  for (int q = 1; q <= b->ccblocks; q++) {
    int nb = b->cc_nph[q], rinx = b->cc_rlen[q];
    if (nb * rinx == 0) continue;
    dgemm_('N', 'T', rinx, rinx, nb, 1.0, LCC + b->cc_off[q - 1], rinx, RCC + b->cc_off[q - 1], rinx, 0.0,
           WCC + b->wcc_off[q - 1], rinx);
  }
#define WX(qx, r, c) (WCC[b->wcc_off[(qx)-1] + ((long)(r)-1) + ((long)(c)-1) * b->cc_rlen[qx]])
#pragma omp parallel for schedule(dynamic)
  for (int q = 1; q <= b->nblocks; q++) {
    int Jtot = b->blk[q - 1].J2;
    for (int g = 1; g <= 6; g++) {
      int n1 = b->blk[q - 1].gam[g - 1].n1, n2 = b->blk[q - 1].gam[g - 1].n2;
      if (n1 * n2 == 0) continue;
      int c1 = sea1[g - 1], c2 = sea2[g - 1], square = sqs[g - 1], jxstart = jst[g - 1];
      for (int IX = 1; IX <= n1; IX++) {
        double pre = 1.0;
        int i = QN(b, q, c1, IX, 1), j = QN(b, q, c1, IX, 2);
        if (i == j) pre = .70710678118;
        int ji = b->jj[i], jj = b->jj[j], li = b->ll[i], lj = b->ll[j], ti = b->itzp[i], tj = b->itzp[j];
        for (int JX = imin_(jxstart, IX); JX <= n2; JX++) {
          double pre2 = 1.0;
          int k = QN(b, q, c2, JX, 1), l = QN(b, q, c2, JX, 2);
          if (k == l) pre2 = .70710678118;
          int jk = b->jj[k], jl = b->jj[l], lk = b->ll[k], ll = b->ll[l], tk = b->itzp[k], tl = b->itzp[l];
          double sm = 0.0;
          int jmin = imax_(iabs_(jj - jl), iabs_(ji - jk));
          int jmax = imin_(jj + jl, ji + jk);
          int Tz = iabs_(ti - tk) / 2;
          if (iabs_(tl - tj) != Tz * 2) continue;
          int PAR = imod_(li + lk, 2);
          if (imod_(ll + lj, 2) != PAR) continue;
          double phase = ipow_m1((ji + jj + jk + jl) / 2);
          for (int JP = jmin; JP <= jmax; JP += 2) {
            int qx = JP / 2 + 1 + Tz * (JTM + 1) + 2 * PAR * (JTM + 1);
            int rjl = cc_rval(b, j, l, qx), rik = cc_rval(b, i, k, qx);
            int gjl = cc_rval(b, l, j, qx), gik = cc_rval(b, k, i, qx);
            sm = sm - ipow_m1((jl + jk + Jtot) / 2) *
                          ((WX(qx, gik, rjl) + phase * WX(qx, gjl, rik)) * hL -
                           (phase * WX(qx, rik, gjl) + WX(qx, rjl, gik)) * hR) *
                          sixj(b, ji, jj, Jtot, jl, jk, JP);
          }
          Tz = iabs_(ti - tl) / 2;
          if (iabs_(tk - tj) != Tz * 2) continue;
          PAR = imod_(li + ll, 2);
          if (imod_(lk + lj, 2) != PAR) continue;
          jmin = imax_(iabs_(ji - jl), iabs_(jj - jk));
          jmax = imin_(ji + jl, jj + jk);
          phase = ipow_m1((ji + jj + jk + jl) / 2);
          for (int JP = jmin; JP <= jmax; JP += 2) {
            int qx = JP / 2 + 1 + Tz * (JTM + 1) + 2 * PAR * (JTM + 1);
            int ril = cc_rval(b, i, l, qx), rjk = cc_rval(b, j, k, qx);
            int gil = cc_rval(b, l, i, qx), gjk = cc_rval(b, k, j, qx);
            sm = sm + ((WX(qx, gil, rjk) + phase * WX(qx, gjk, ril)) * hL -
                       (phase * WX(qx, ril, gjk) + WX(qx, rjk, gil)) * hR) *
                          sixj(b, ji, jj, Jtot, jk, jl, JP);
          }
          GX(b, RES, q, g, IX, JX) = GX(b, RES, q, g, IX, JX) + sm * pre * pre2;
          if (square) GX(b, RES, q, g, JX, IX) = GX(b, RES, q, g, IX, JX) * hRES;
        }
      }
    }
  }
#undef WX
}

/* Work buffers for one commutator: w1, w2 (operators), LCC, RCC, WCC. */
typedef struct {
  double *w1, *w2, *LCC, *RCC, *WCC;
} owork;

static owork work_new(const obasis *b) {
  owork w;
  w.w1 = calloc(b->nfull, sizeof(double));
  w.w2 = calloc(b->nfull, sizeof(double));
  w.LCC = calloc(b->cc_total + 1, sizeof(double));
  w.RCC = calloc(b->cc_total + 1, sizeof(double));
  w.WCC = calloc(b->wcc_total + 1, sizeof(double));
  return w;
}
static void work_free(owork *w) {
  free(w->w1); free(w->w2); free(w->LCC); free(w->RCC); free(w->WCC);
}

/* The commutator sequence of IMSRG_MAGNUS.f90:207-219 (with_e0) and
 * :676-685 (without E0; RES%E0 is left as it was). */
static void commutator_seq(const obasis *b, const double *L, int hL, const double *R, int hR, double *RES, int hRES,
                           int with_e0, owork *w) {
  orc_cross_coupled(b, R, hR, w->RCC);
  orc_cross_coupled(b, L, hL, w->LCC);
  if (with_e0) RES[0] = orc_comm110(b, L, hL, R, hR) + orc_comm220(b, L, hL, R, hR);
  comm111(b, L, hL, R, hR, RES);
  comm121(b, L, hL, R, hR, RES, hRES);
  comm122(b, L, hL, R, hR, RES, hRES);
  comm222_pphh(b, L, hL, R, hR, RES, w->w1, w->w2);
  comm221(b, hL, hR, RES, hRES, w->w1, w->w2);
  comm222_ph(b, w->LCC, hL, w->RCC, hR, RES, hRES, w->WCC);
}

/* Full [L,R] into RES with RES%herm = -hL*hR (brute_force_testing.f90:509-532).
 * RES is overwritten (E0 = 110 + 220). */
void orc_commutator(const obasis *b, const double *L, int hL, const double *R, int hR, double *RES) {
  owork w = work_new(b);
  memset(RES, 0, b->nfull * sizeof(double));
  commutator_seq(b, L, hL, R, hR, RES, -hL * hR, 1, &w);
  work_free(&w);
}

/* Intermediates of one commutator, for fine-grained parity tests. */
void orc_commutator_parts(const obasis *b, const double *L, int hL, const double *R, int hR, double *RES,
                          double *w1, double *w2, double *LCC, double *RCC, double *WCC) {
  owork w = work_new(b);
  memset(RES, 0, b->nfull * sizeof(double));
  commutator_seq(b, L, hL, R, hR, RES, -hL * hR, 1, &w);
  memcpy(w1, w.w1, b->nfull * sizeof(double));
  memcpy(w2, w.w2, b->nfull * sizeof(double));
  memcpy(LCC, w.LCC, b->cc_total * sizeof(double));
  memcpy(RCC, w.RCC, b->cc_total * sizeof(double));
  memcpy(WCC, w.WCC, b->wcc_total * sizeof(double));
  work_free(&w);
}

/* ------------------------------------------------------------------ */
/* Generators: White (generators.f90:4-106), atan (:162-266), atanxx  */
/* (:271-376; denominators from Hold, numerators from H), w2 (:109-159) */
/* ------------------------------------------------------------------ */
static void gen_core(const obasis *b, const double *Hd, int hd, const double *Hn, double *ETA, int use_atan) {
  /* ETA%fpp = 0, ETA%fhh = 0; fph entries with mismatched (l,j,tz) keep
   * their previous value in the reference; callers pass a zeroed ETA. */
  for (long i = 0; i < (long)b->P * b->P; i++) ETA[b->off_fpp + i] = 0.0;
  for (long i = 0; i < (long)b->A * b->A; i++) ETA[b->off_fhh + i] = 0.0;
  for (int a = 1; a <= b->P; a++) {
    int ak = b->parts[a];
    int ja = b->jj[ak], la = b->ll[ak], ta = b->itzp[ak];
    for (int i = 1; i <= b->A; i++) {
      int ik = b->holes[i];
      int ji = b->jj[ik], li = b->ll[ik], ti = b->itzp[ik];
      if (ji != ja || li != la || ti != ta) continue;
      double Eden = 0.0;
      for (int JT = 0; JT <= 2 * ji; JT += 2) Eden = Eden - (JT + 1) * v_elem(b, ak, ik, ak, ik, JT, Hd, hd);
      Eden = Eden / (ji + 1.0) / (ji + 1.0);
      Eden = Eden + FPP(b, Hd, a, a) - FHH(b, Hd, i, i);
      FPH(b, ETA, a, i) = use_atan ? atan(2 * FPH(b, Hn, a, i) / Eden) * 0.5 : FPH(b, Hn, a, i) / Eden;
    }
  }
  for (int q = 1; q <= b->nblocks; q++) {
    const oblock *B = &b->blk[q - 1];
    for (int g = 1; g <= 6; g++) memset(GAM(b, ETA, q, g), 0, (long)B->gam[g - 1].n1 * B->gam[g - 1].n2 * sizeof(double));
    for (int IX = 1; IX <= B->npp; IX++) {
      int a = QN(b, q, 1, IX, 1), bb = QN(b, q, 1, IX, 2);
      int ja = b->jj[a], jb = b->jj[bb];
      for (int JX = 1; JX <= B->nhh; JX++) {
        int i = QN(b, q, 3, JX, 1), j = QN(b, q, 3, JX, 2);
        int ji = b->jj[i], jj = b->jj[j];
        double Eden = 0.0;
        Eden = Eden + twobody_monopole(b, a, bb, ja, jb, Hd, hd);
        Eden = Eden + twobody_monopole(b, i, j, ji, jj, Hd, hd);
        Eden = Eden - twobody_monopole(b, a, i, ja, ji, Hd, hd);
        Eden = Eden - twobody_monopole(b, a, j, ja, jj, Hd, hd);
        Eden = Eden - twobody_monopole(b, i, bb, ji, jb, Hd, hd);
        Eden = Eden - twobody_monopole(b, j, bb, jj, jb, Hd, hd);
        Eden = Eden + f_elem(b, a, a, Hd, hd) + f_elem(b, bb, bb, Hd, hd) - f_elem(b, i, i, Hd, hd) -
               f_elem(b, j, j, Hd, hd);
        GX(b, ETA, q, 3, IX, JX) =
            use_atan ? 0.5 * atan(2 * GX(b, Hn, q, 3, IX, JX) / Eden) : GX(b, Hn, q, 3, IX, JX) / Eden;
      }
    }
  }
}

void orc_white(const obasis *b, const double *H, int hH, double *ETA) { gen_core(b, H, hH, H, ETA, 0); }

void orc_atan(const obasis *b, const double *H, int hH, double *ETA) { gen_core(b, H, hH, H, ETA, 1); }

void orc_atanxx(const obasis *b, const double *Hold, int hold, const double *H, double *ETA) {
  gen_core(b, Hold, hold, H, ETA, 1);
}

/* build_gs_w2: ETA1 = atan(H); H2 = [ETA1, H]; ETA2 = atanxx(H, H2);
 * ETA = 1.5 ETA1 + 0.5 ETA2 (fresh, zeroed work operators). */
void orc_w2(const obasis *b, const double *H, int hH, double *ETA) {
  double *E1 = calloc(b->nfull, sizeof(double)), *E2 = calloc(b->nfull, sizeof(double)),
         *H2 = calloc(b->nfull, sizeof(double));
  orc_atan(b, H, hH, E1);
  orc_commutator(b, E1, -1, H, hH, H2);
  orc_atanxx(b, H, hH, H2, E2);
  orc_add(b, E1, 1.5, E2, 0.5, ETA);
  free(E1); free(E2); free(H2);
}

static void generator(const obasis *b, int gen, const double *H, double *ETA) {
  memset(ETA, 0, b->nfull * sizeof(double));
  if (gen == 1) orc_atan(b, H, 1, ETA);
  else if (gen == 2) orc_w2(b, H, 1, ETA);
  else orc_white(b, H, 1, ETA);
}

/* ------------------------------------------------------------------ */
/* normal ordering, basic_IMSRG.f90:2375-2506                          */
/* ------------------------------------------------------------------ */
void orc_normal_order(const obasis *b, double *H, int herm) {
  double *T = malloc(b->nfull * sizeof(double));
  memcpy(T, H, b->nfull * sizeof(double));
  double sm = 0.0;
  for (int i = 1; i <= b->norb; i++) sm += f_elem(b, i, i, T, herm) * b->con[i] * (b->jj[i] + 1);
  sm = sm * 2.0;
  for (int i = 1; i <= b->norb; i++)
    for (int j = 1; j <= b->norb; j++) {
      if (b->con[i] * b->con[j] == 0) continue;
      for (int JT = iabs_(b->jj[i] - b->jj[j]); JT <= b->jj[i] + b->jj[j]; JT += 2)
        sm += v_elem(b, i, j, i, j, JT, T, herm) * (JT + 1);
    }
  H[0] = sm * 0.5;
  /* pass 0: fhh (a hole, b>=a hole); 1: fph (a part, b hole); 2: fpp (a part, b>=a part) */
  for (int pass = 0; pass < 3; pass++) {
    int na = (pass == 0) ? b->A : b->P;
    int nbb = (pass == 2) ? b->P : b->A;
    for (int a = 1; a <= na; a++) {
      int blo = (pass == 1) ? 1 : a;
      for (int bb = blo; bb <= nbb; bb++) {
        int ax = (pass == 0) ? b->holes[a] : b->parts[a];
        int bx = (pass == 2) ? b->parts[bb] : b->holes[bb];
        if (b->jj[ax] != b->jj[bx] || b->ll[ax] != b->ll[bx] || b->itzp[ax] != b->itzp[bx]) continue;
        double s = 0.0;
        for (int i = 1; i <= b->A; i++) {
          int ix = b->holes[i];
          for (int JT = iabs_(b->jj[ix] - b->jj[ax]); JT <= b->jj[ix] + b->jj[ax]; JT += 2)
            s += (JT + 1.0) / (b->jj[ax] + 1) * v_elem(b, ax, ix, bx, ix, JT, T, herm);
        }
        double v = f_elem(b, ax, bx, T, herm) + s;
        if (pass == 0) {
          FHH(b, H, a, bb) = v;
          FHH(b, H, bb, a) = v;
        } else if (pass == 1) {
          FPH(b, H, a, bb) = v;
        } else {
          FPP(b, H, a, bb) = v;
          FPP(b, H, bb, a) = v;
        }
      }
    }
  }
  free(T);
}

/* ------------------------------------------------------------------ */
/* vectorize / repackage, basic_IMSRG.f90:3794-3918                    */
/* ------------------------------------------------------------------ */
void orc_vectorize(const obasis *b, const double *op, double *v) {
  long k = 0;
  v[k++] = op[0];
  for (int i = 1; i <= b->A; i++)
    for (int j = 1; j <= b->A; j++) v[k++] = FHH(b, op, j, i);
  for (int i = 1; i <= b->P; i++)
    for (int j = 1; j <= b->P; j++) v[k++] = FPP(b, op, j, i);
  for (int i = 1; i <= b->A; i++)
    for (int j = 1; j <= b->P; j++) v[k++] = FPH(b, op, j, i);
  for (int l = 1; l <= b->nblocks; l++)
    for (int g = 1; g <= 6; g++) {
      int n1 = b->blk[l - 1].gam[g - 1].n1, n2 = b->blk[l - 1].gam[g - 1].n2;
      for (int i = 1; i <= n2; i++)
        for (int j = imin_(jst[g - 1], i); j <= n1; j++) v[k++] = GX(b, op, l, g, j, i);
    }
}

void orc_repackage(const obasis *b, const double *v, int herm, double *op) {
  long k = 0;
  op[0] = v[k++];
  for (int i = 1; i <= b->A; i++)
    for (int j = 1; j <= b->A; j++) FHH(b, op, j, i) = v[k++];
  for (int i = 1; i <= b->P; i++)
    for (int j = 1; j <= b->P; j++) FPP(b, op, j, i) = v[k++];
  for (int i = 1; i <= b->A; i++)
    for (int j = 1; j <= b->P; j++) FPH(b, op, j, i) = v[k++];
  for (int l = 1; l <= b->nblocks; l++)
    for (int g = 1; g <= 6; g++) {
      int n1 = b->blk[l - 1].gam[g - 1].n1, n2 = b->blk[l - 1].gam[g - 1].n2;
      for (int i = 1; i <= n2; i++)
        for (int j = imin_(jst[g - 1], i); j <= n1; j++) {
          GX(b, op, l, g, j, i) = v[k];
          if (sqs[g - 1]) GX(b, op, l, g, i, j) = v[k] * herm;
          k++;
        }
    }
}

/* ------------------------------------------------------------------ */
/* Magnus flow, IMSRG_MAGNUS.f90                                       */
/* ------------------------------------------------------------------ */
static const double magnus_cof[7] = {1.0, -0.5, .0833333333, 0.0, -0.00138888888, 0.0, 3.306878e-5};

/* MAGNUS_EXPAND, IMSRG_MAGNUS.f90:622-693: DG (in: eta, out: dOmega/ds).
 * Returns the number of commutators evaluated. */
int orc_magnus_expand(const obasis *b, double *DG, const double *G) {
  const double conv = 1e-6;
  owork w = work_new(b);
  double *INT1 = calloc(b->nfull, sizeof(double)), *INT2 = calloc(b->nfull, sizeof(double)),
         *AD = calloc(b->nfull, sizeof(double));
  double advals[8] = {0};
  int ncomm = 0;
  memcpy(INT2, DG, b->nfull * sizeof(double));
  advals[1] = orc_norm(b, INT2);
  double fullnorm = orc_norm(b, G);
  if (fullnorm < 1e-9) goto done;
  int q = 1;
  for (int i = 2; i <= 7; i++) {
    memcpy(INT1, DG, b->nfull * sizeof(double));
    memcpy(AD, INT2, b->nfull * sizeof(double));
    double adnorm = advals[i - q];
    q = (fabs(magnus_cof[i - 1]) > 1e-6) ? 1 : 2;
    if (fabs(adnorm / fullnorm) < conv) break;
    commutator_seq(b, G, -1, AD, -1, INT2, -1, 0, &w);
    ncomm++;
    orc_add(b, INT1, 1.0, INT2, magnus_cof[i - 1], DG);
    advals[i] = orc_norm(b, INT2) * fabs(magnus_cof[i - 1]);
  }
done:
  free(INT1); free(INT2); free(AD);
  work_free(&w);
  return ncomm;
}

/* BCH_EXPAND, IMSRG_MAGNUS.f90:149-234: HS = e^G H e^-G.  Returns the number
 * of commutators, or -1 when 39 terms did not converge ("clipping BCH"). */
int orc_bch_expand(const obasis *b, double *HS, const double *G, const double *H) {
  const double conv = 1e-6;
  owork w = work_new(b);
  double *INT1 = calloc(b->nfull, sizeof(double)), *INT2 = calloc(b->nfull, sizeof(double)),
         *AD = calloc(b->nfull, sizeof(double));
  double coef = 1.0;
  int ncomm = 0, iw;
  memcpy(HS, H, b->nfull * sizeof(double));
  memcpy(INT2, HS, b->nfull * sizeof(double));
  for (iw = 2; iw <= 40; iw++) {
    coef = coef / (iw - 1.0);
    memcpy(INT1, HS, b->nfull * sizeof(double));
    memcpy(AD, INT2, b->nfull * sizeof(double));
    memset(INT2, 0, b->nfull * sizeof(double));
    commutator_seq(b, G, -1, AD, 1, INT2, 1, 1, &w);
    ncomm++;
    orc_add(b, INT1, 1.0, INT2, coef, HS);
    double adv = orc_norm(b, INT2) * coef;
    if (adv < conv) break;
  }
  free(INT1); free(INT2); free(AD);
  work_free(&w);
  return (iw > 40) ? -1 : ncomm;
}

/* magnus_decouple, IMSRG_MAGNUS.f90:15-128, White generator, with an added
 * stop at s >= s_max.  trace[5*k..] = (step, s, E0, E0+mbpt2, |mbpt2|) for
 * k = 0..nsteps; returns the number of steps (or -1 on BCH clipping).
 * HS: in = normal-ordered H, out = H(s).  G: out = Omega(s). */
int orc_magnus_decouple_gen(const obasis *b, int gen, double *HS, double *G, double s_max, double ds,
                            int max_steps, double *trace, int *ncomm_total) {
  double *H = malloc(b->nfull * sizeof(double)), *DG = calloc(b->nfull, sizeof(double));
  memset(G, 0, b->nfull * sizeof(double));
  generator(b, gen, HS, DG);
  memcpy(H, HS, b->nfull * sizeof(double));
  double s = 0.0;
  double E_mbpt2 = orc_mbpt2(b, HS, 1);
  double crit = fabs(E_mbpt2);
  int steps = 0, nct = 0;
  trace[0] = 0; trace[1] = s; trace[2] = HS[0]; trace[3] = HS[0] + E_mbpt2; trace[4] = crit;
  while (crit > 1e-6 && s < s_max - 1e-12 && steps < max_steps) {
    steps++;
    nct += orc_magnus_expand(b, DG, G);
    orc_add(b, G, 1.0, DG, ds, G); /* euler_step, IMSRG_MAGNUS.f90:756-766 */
    s = s + ds;
    int nb = orc_bch_expand(b, HS, G, H);
    if (nb < 0) { steps = -1; break; }
    nct += nb;
    generator(b, gen, HS, DG);
    E_mbpt2 = orc_mbpt2(b, HS, 1);
    crit = fabs(E_mbpt2);
    double *t = trace + 5 * steps;
    t[0] = steps; t[1] = s; t[2] = HS[0]; t[3] = HS[0] + E_mbpt2; t[4] = crit;
  }
  if (ncomm_total) *ncomm_total = nct;
  free(H); free(DG);
  return steps;
}

int orc_magnus_decouple(const obasis *b, double *HS, double *G, double s_max, double ds, int max_steps,
                        double *trace, int *ncomm_total) {
  return orc_magnus_decouple_gen(b, 0, HS, G, s_max, ds, max_steps, trace, ncomm_total);
}

/* ------------------------------------------------------------------ */
/* brute-force known-answer formulas, brute_force_testing.f90          */
/* ------------------------------------------------------------------ */
/* brute_force_testing.f90:1887-1928 */
double orc_bf_0body(const obasis *b, const double *AA, int hA, const double *BB, int hB) {
  int JTM = b->Jtotal_max * 2, N = b->norb;
  double sm = 0.0;
  for (int i = 1; i <= N; i++) {
    int ji = b->jj[i];
    for (int j = 1; j <= N; j++)
      sm += (b->con[i] - b->con[j]) * (ji + 1.0) * f_elem(b, i, j, AA, hA) * f_elem(b, j, i, BB, hB);
  }
  for (int i = 1; i <= N; i++)
    for (int j = 1; j <= N; j++)
      for (int k = 1; k <= N; k++)
        for (int l = 1; l <= N; l++) {
          int w = b->con[i] * b->con[j] * (1 - b->con[k]) * (1 - b->con[l]) -
                  b->con[k] * b->con[l] * (1 - b->con[i]) * (1 - b->con[j]);
          if (w == 0) continue;
          for (int Jt = 0; Jt <= JTM; Jt += 2)
            sm += w * (Jt + 1.0) * v_elem(b, i, j, k, l, Jt, AA, hA) * v_elem(b, k, l, i, j, Jt, BB, hB) / 4.0;
        }
  return sm;
}

/* brute_force_testing.f90:1765-1823; a, b are orbit indices (1-based) */
double orc_bf_1body(const obasis *b, const double *AA, int hA, const double *BB, int hB, int a, int bo) {
  int JTM = b->Jtotal_max * 2, N = b->norb;
  double sm = 0.0;
  int ja = b->jj[a], jb = b->jj[bo];
  for (int i = 1; i <= N; i++)
    sm += f_elem(b, a, i, AA, hA) * f_elem(b, i, bo, BB, hB) - f_elem(b, a, i, BB, hB) * f_elem(b, i, bo, AA, hA);
  if (ja == jb) {
    for (int i = 1; i <= N; i++)
      for (int j = 1; j <= N; j++) {
        if (b->con[i] == b->con[j]) continue;
        for (int Jt = 0; Jt <= JTM; Jt += 2)
          sm += (b->con[i] - b->con[j]) * (Jt + 1.0) / (ja + 1.0) *
                (f_elem(b, i, j, AA, hA) * v_elem(b, j, a, i, bo, Jt, BB, hB) -
                 f_elem(b, i, j, BB, hB) * v_elem(b, j, a, i, bo, Jt, AA, hA));
      }
    for (int i = 1; i <= N; i++)
      for (int j = 1; j <= N; j++)
        for (int k = 1; k <= N; k++) {
          int w = b->con[i] * b->con[j] * (1 - b->con[k]) + (1 - b->con[i]) * (1 - b->con[j]) * b->con[k];
          if (w == 0) continue;
          for (int Jt = 0; Jt <= JTM; Jt += 2)
            sm += w * (Jt + 1.0) / (ja + 1.0) *
                  (v_elem(b, a, k, i, j, Jt, AA, hA) * v_elem(b, i, j, bo, k, Jt, BB, hB) -
                   v_elem(b, a, k, i, j, Jt, BB, hB) * v_elem(b, i, j, bo, k, Jt, AA, hA)) /
                  2.0;
        }
  }
  return sm;
}

/* brute_force_testing.f90:1975-2076 */
double orc_bf_2body(const obasis *b, const double *AA, int hA, const double *BB, int hB, int a, int bo, int c, int d,
                    int Jtot) {
  int JTM = b->Jtotal_max * 2, N = b->norb;
  double sm = 0.0;
  int ja = b->jj[a], jb = b->jj[bo], jc = b->jj[c], jd = b->jj[d];
  for (int i = 1; i <= N; i++) {
    sm += f_elem(b, a, i, AA, hA) * v_elem(b, i, bo, c, d, Jtot, BB, hB) +
          f_elem(b, bo, i, AA, hA) * v_elem(b, a, i, c, d, Jtot, BB, hB) -
          f_elem(b, i, c, AA, hA) * v_elem(b, a, bo, i, d, Jtot, BB, hB) -
          f_elem(b, i, d, AA, hA) * v_elem(b, a, bo, c, i, Jtot, BB, hB);
    sm += -f_elem(b, a, i, BB, hB) * v_elem(b, i, bo, c, d, Jtot, AA, hA) -
          f_elem(b, bo, i, BB, hB) * v_elem(b, a, i, c, d, Jtot, AA, hA) +
          f_elem(b, i, c, BB, hB) * v_elem(b, a, bo, i, d, Jtot, AA, hA) +
          f_elem(b, i, d, BB, hB) * v_elem(b, a, bo, c, i, Jtot, AA, hA);
  }
  for (int i = 1; i <= N; i++)
    for (int j = 1; j <= N; j++)
      sm += 0.5 * (1 - b->con[i] - b->con[j]) *
            (v_elem(b, a, bo, i, j, Jtot, AA, hA) * v_elem(b, i, j, c, d, Jtot, BB, hB) -
             v_elem(b, a, bo, i, j, Jtot, BB, hB) * v_elem(b, i, j, c, d, Jtot, AA, hA));
  for (int i = 1; i <= N; i++) {
    int ji = b->jj[i];
    for (int j = 1; j <= N; j++) {
      int jj = b->jj[j];
      if (b->con[i] - b->con[j] == 0) continue;
      for (int J1 = 0; J1 <= JTM; J1 += 2)
        for (int J2 = 0; J2 <= JTM; J2 += 2) {
          double t = ipow_m1((J1 + J2 + ja - jc) / 2) * (J1 + 1.0) * (J2 + 1.0) *
                         coef9(b, jj, J1, ja, J2, ji, jb, jc, jd, Jtot) * v_elem(b, j, a, i, d, J1, AA, hA) *
                         v_elem(b, i, bo, j, c, J2, BB, hB) -
                     ipow_m1((J1 + J2 + jb - jc) / 2) * (J1 + 1.0) * (J2 + 1.0) *
                         coef9(b, jj, J1, jb, J2, ji, ja, jc, jd, Jtot) * v_elem(b, j, bo, i, d, J1, AA, hA) *
                         v_elem(b, i, a, j, c, J2, BB, hB) * ipow_m1((ja + jb - Jtot) / 2) -
                     ipow_m1((J1 + J2 + ja - jd) / 2) * (J1 + 1.0) * (J2 + 1.0) *
                         coef9(b, jj, J1, ja, J2, ji, jb, jd, jc, Jtot) * v_elem(b, j, a, i, c, J1, AA, hA) *
                         v_elem(b, i, bo, j, d, J2, BB, hB) * ipow_m1((jc + jd - Jtot) / 2) +
                     ipow_m1((J1 + J2 + jb - jd) / 2) * (J1 + 1.0) * (J2 + 1.0) *
                         coef9(b, jj, J1, jb, J2, ji, ja, jd, jc, Jtot) * v_elem(b, j, bo, i, c, J1, AA, hA) *
                         v_elem(b, i, a, j, d, J2, BB, hB) * ipow_m1((ja + jb + jc + jd) / 2);
          sm += (b->con[i] - b->con[j]) * t;
        }
    }
  }
  return sm;
}

/* ------------------------------------------------------------------ */
/* exported accessors for the Python test harness                      */
/* ------------------------------------------------------------------ */
/* info: norb, A, P, nblocks, Jtotal_max, lmax, nfull, neq, ccblocks, cc_total, wcc_total */
void orc_basis_info(const obasis *b, long *info) {
  info[0] = b->norb; info[1] = b->A; info[2] = b->P; info[3] = b->nblocks; info[4] = b->Jtotal_max;
  info[5] = b->lmax; info[6] = b->nfull; info[7] = b->neq; info[8] = b->ccblocks; info[9] = b->cc_total;
  info[10] = b->wcc_total;
}

/* per block: J2, par, tz, npp, nph, nhh */
void orc_block_dims(const obasis *b, int *out) {
  for (int q = 0; q < b->nblocks; q++) {
    out[6 * q + 0] = b->blk[q].J2; out[6 * q + 1] = b->blk[q].par; out[6 * q + 2] = b->blk[q].tz;
    out[6 * q + 3] = b->blk[q].npp; out[6 * q + 4] = b->blk[q].nph; out[6 * q + 5] = b->blk[q].nhh;
  }
}

/* pair list of category c (1 pp, 2 ph, 3 hh) of block q (1-based) */
void orc_block_qn(const obasis *b, int q, int c, int *out) {
  const oblock *B = &b->blk[q - 1];
  int n = (c == 1) ? B->npp : (c == 2) ? B->nph : B->nhh;
  for (int i = 0; i < 2 * n; i++) out[i] = B->qn[c - 1][i];
}

/* per CC block: J2, nph, rlen */
void orc_cc_dims(const obasis *b, int *out) {
  for (int q = 1; q <= b->ccblocks; q++) {
    out[3 * (q - 1)] = b->cc_J2[q]; out[3 * (q - 1) + 1] = b->cc_nph[q]; out[3 * (q - 1) + 2] = b->cc_rlen[q];
  }
}

double orc_v_elem(const obasis *b, int a, int bb, int c, int d, int J, const double *op, int herm) {
  return v_elem(b, a, bb, c, d, J, op, herm);
}
double orc_f_elem(const obasis *b, int a, int bb, const double *op, int herm) { return f_elem(b, a, bb, op, herm); }
double orc_sixj(const obasis *b, int j1, int j2, int j3, int j4, int j5, int j6) {
  return sixj(b, j1, j2, j3, j4, j5, j6);
}
double orc_d6ji(const obasis *b, int j1, int j2, int j3, int j4, int j5, int j6) {
  return d6ji(b, j1, j2, j3, j4, j5, j6);
}
double orc_coef9(const obasis *b, int j1, int j2, int j3, int j4, int j5, int j6, int j7, int j8, int j9) {
  return coef9(b, j1, j2, j3, j4, j5, j6, j7, j8, j9);
}
void orc_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}
int orc_get_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
