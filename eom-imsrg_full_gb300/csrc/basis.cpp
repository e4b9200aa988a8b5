// basis.cpp -- host construction of the basis tables and their device copies.
//
// Restates the layout routines of n-parzuchowski/EOM-IMSRG_FULL (im-SRG/):
//   holes / particles, hb4 / pb4          basic_IMSRG.f90:380-398
//   (2J,Tz,parity) blocks, qn, xmap       basic_IMSRG.f90:477-641
//   jbas%states (same (l,j,tz) orbits)    basic_IMSRG.f90:302-340
//   cross-coupled blocks, rmap/nbmap      cross_coupled.f90:61-177
//   6j table                              basic_IMSRG.f90:2183-2288 (values from
//                                         the Racah formula, anglib.f:285-377)
//   vectorize order                       basic_IMSRG.f90:3794-3918
// and lays them out as dense device tables (pair -> row, (block,i,j) -> CC
// row) in place of the reference's linear searches.
#include <cmath>
#include <cstring>
#include <algorithm>
#include <map>

#include "internal.h"

namespace imsrg {

int cuda_status(cudaError_t e) {
  if (e == cudaSuccess) return IMSRG_OK;
  if (e == cudaErrorMemoryAllocation) return IMSRG_ERR_OOM;
  if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) return IMSRG_ERR_NO_DEVICE;
  return IMSRG_ERR_CUDA;
}

namespace {

bool tri(int j1, int j2, int J) { return J <= j1 + j2 && J >= std::abs(j1 - j2); }

// {a b c; d e f} with doubled arguments by the Racah single sum, long double.
struct SixJ {
  long double fact[256];
  SixJ() {
    fact[0] = 1.0L;
    for (int i = 1; i < 256; i++) fact[i] = fact[i - 1] * (long double)i;
  }
  long double delta(int a, int b, int c) const {  // doubled
    return std::sqrt(fact[(a + b - c) / 2] * fact[(a - b + c) / 2] * fact[(-a + b + c) / 2] /
                     fact[(a + b + c) / 2 + 1]);
  }
  double operator()(int a, int b, int c, int d, int e, int f) const {
    auto ok = [](int x, int y, int z) { return tri(x, y, z) && ((x + y + z) % 2 == 0); };
    if (a < 0 || b < 0 || c < 0 || d < 0 || e < 0 || f < 0) return 0.0;
    if (!(ok(a, b, c) && ok(a, e, f) && ok(d, b, f) && ok(d, e, c))) return 0.0;
    int s1 = (a + b + c) / 2, s2 = (a + e + f) / 2, s3 = (d + b + f) / 2, s4 = (d + e + c) / 2;
    int p1 = (a + b + d + e) / 2, p2 = (b + c + e + f) / 2, p3 = (c + a + f + d) / 2;
    int tmin = std::max(std::max(s1, s2), std::max(s3, s4));
    int tmax = std::min(std::min(p1, p2), p3);
    long double sum = 0.0L;
    for (int t = tmin; t <= tmax; t++) {
      long double term = fact[t + 1] / (fact[t - s1] * fact[t - s2] * fact[t - s3] * fact[t - s4] *
                                        fact[p1 - t] * fact[p2 - t] * fact[p3 - t]);
      sum += (t % 2) ? -term : term;
    }
    return (double)(sum * delta(a, b, c) * delta(a, e, f) * delta(d, b, f) * delta(d, e, c));
  }
};

template <typename T>
int dev_upload(imsrg_basis *b, const std::vector<T> &h, const T **out) {
  size_t n = std::max<size_t>(h.size(), 1) * sizeof(T);
  void *p = nullptr;
  IMSRG_CUDA_TRY(cudaMalloc(&p, n));
  b->dev_allocs.push_back(p);
  if (!h.empty()) IMSRG_CUDA_TRY(cudaMemcpy(p, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice));
  *out = (const T *)p;
  return IMSRG_OK;
}

int dev_alloc(imsrg_basis *b, size_t bytes, void **out) {
  void *p = nullptr;
  IMSRG_CUDA_TRY(cudaMalloc(&p, std::max<size_t>(bytes, 16)));
  IMSRG_CUDA_TRY(cudaMemset(p, 0, std::max<size_t>(bytes, 16)));
  b->dev_allocs.push_back(p);
  *out = p;
  return IMSRG_OK;
}

// --- grouped GEMM problems of commutator_222_pp_hh (commutators.f90:596-766)
// and of the WCC product of commutator_222_ph (:792-802).
struct ProbBuilder {
  std::vector<GemmProb> probs;
  void add(int M, int N, int K, int c_dst, long c_off, int ldc, std::initializer_list<GemmTerm> terms) {
    if (M <= 0 || N <= 0) return;
    GemmProb p{};
    p.M = M;
    p.N = N;
    p.K = K;
    p.nterms = 0;
    for (const GemmTerm &t : terms) p.t[p.nterms++] = t;
    p.c_dst = c_dst;
    p.c_off = c_off;
    p.ldc = ldc;
    probs.push_back(p);
  }
};

GemmTerm term(int a, long aoff, int lda, int ta, int bsrc, long boff, int ldb, int tb, double coef, int hl = 0,
              int hr = 0) {
  GemmTerm t{};
  t.a_src = a;
  t.a_off = aoff;
  t.lda = lda;
  t.ta = ta;
  t.b_src = bsrc;
  t.b_off = boff;
  t.ldb = ldb;
  t.tb = tb;
  t.coef = coef;
  t.use_hl = hl;
  t.use_hr = hr;
  return t;
}

}  // namespace

double sixj(int a, int b, int c, int d, int e, int f) {
  static const SixJ sj;
  return sj(a, b, c, d, e, f);
}

// Host restatement of the element location of v_elem (basic_IMSRG.f90:
// 1270-1385): the stored element that <a bb|V|c d>_J reads, with the
// pair-reordering phase, the sqrt(2) factors of identical-orbit pairs and
// whether it is read transposed (times herm).
HLoc v_location(const imsrg_basis *b, int a, int bb, int c, int d, int J2) {
  const int N = b->norb, nJ = b->jtm + 1;
  HLoc r{-1, 0, 0, 0};
  if (!(tri(b->jj[a], b->jj[bb], J2) && tri(b->jj[c], b->jj[d], J2))) return r;
  int Pp = (b->ll[a] + b->ll[bb]) & 1;
  if (((b->ll[c] + b->ll[d]) & 1) != Pp) return r;
  int tz2 = b->itzp[a] + b->itzp[bb];
  if (b->itzp[c] + b->itzp[d] != tz2) return r;
  int qq = 3 * J2 + 2 * (tz2 / 2 + 1) + Pp;
  int C1 = b->con[a] + b->con[bb] + 1, C2 = b->con[c] + b->con[d] + 1;
  int qx = C1 * C2;
  if (qx == 9) qx = 5;
  int i1, i2;
  if (a > bb) {
    i1 = b->pairrow[((size_t)bb * N + a) * nJ + J2 / 2];
    r.neg = (1 + (b->jj[a] + b->jj[bb] - J2) / 2) & 1;
  } else {
    r.nsq += (a == bb);
    i1 = b->pairrow[((size_t)a * N + bb) * nJ + J2 / 2];
  }
  if (c > d) {
    i2 = b->pairrow[((size_t)d * N + c) * nJ + J2 / 2];
    r.neg ^= (1 + (b->jj[c] + b->jj[d] - J2) / 2) & 1;
  } else {
    r.nsq += (c == d);
    i2 = b->pairrow[((size_t)c * N + d) * nJ + J2 / 2];
  }
  int sg = qq * 6 + qx - 1;
  r.trans = C1 > C2;
  r.idx = r.trans ? b->gam_off[sg] + i2 + (long)i1 * b->gam_n1[sg] : b->gam_off[sg] + i1 + (long)i2 * b->gam_n1[sg];
  return r;
}

int build_basis(imsrg_basis *b) {
  const int N = b->norb;
  // holes / particles (find_holes, basic_IMSRG.f90:380-398)
  std::vector<int> orbpos(N);
  b->holes.clear();
  b->parts.clear();
  for (int i = 0; i < N; i++) {
    if (b->con[i] == 1) {
      orbpos[i] = (int)b->holes.size();
      b->holes.push_back(i);
    } else {
      orbpos[i] = (int)b->parts.size();
      b->parts.push_back(i);
    }
  }
  b->A = (int)b->holes.size();
  b->P = (int)b->parts.size();
  b->jtm = *std::max_element(b->jj.begin(), b->jj.end());
  const int jtm = b->jtm, nJ = jtm + 1, nj = (jtm + 1) / 2;
  const int A = b->A, P = b->P;

  // blocks (allocate_blocks, basic_IMSRG.f90:528-637)
  b->nblocks = (jtm + 1) * 6;
  b->npp.assign(b->nblocks, 0);
  b->nph.assign(b->nblocks, 0);
  b->nhh.assign(b->nblocks, 0);
  b->qn.assign(b->nblocks * 3, {});
  b->gam_off.assign(b->nblocks * 6, 0);
  b->gam_n1.assign(b->nblocks * 6, 0);
  b->gam_n2.assign(b->nblocks * 6, 0);
  b->pairrow.assign((size_t)N * N * nJ, -1);
  std::vector<int> &pairrow = b->pairrow;
  std::vector<int> blk_J2(b->nblocks);
  b->off_fhh = 1;
  b->off_fph = 1 + (long)A * A;
  b->off_fpp = b->off_fph + (long)P * A;
  long off = b->off_fpp + (long)P * P;
  long neq = 1 + (long)A * A + (long)P * P + (long)P * A;
  static const int sq[6] = {1, 0, 0, 1, 1, 0};
  int q = 0;
  for (int J2 = 0; J2 <= 2 * jtm; J2 += 2)
    for (int Tz = -1; Tz <= 1; Tz++)
      for (int Par = 0; Par <= 1; Par++, q++) {
        blk_J2[q] = J2;
        int cnt[3] = {0, 0, 0};
        for (int i = 0; i < N; i++)
          for (int j = i; j < N; j++) {
            if (Tz != (b->itzp[i] + b->itzp[j]) / 2) continue;
            if (Par != (b->ll[i] + b->ll[j]) % 2) continue;
            if (!tri(b->jj[i], b->jj[j], J2)) continue;
            int c = b->con[i] + b->con[j];
            pairrow[((size_t)i * N + j) * nJ + J2 / 2] = cnt[c]++;
            b->qn[q * 3 + c].push_back(i);
            b->qn[q * 3 + c].push_back(j);
          }
        b->npp[q] = cnt[0];
        b->nph[q] = cnt[1];
        b->nhh[q] = cnt[2];
        int d1[6] = {cnt[0], cnt[0], cnt[0], cnt[1], cnt[2], cnt[1]};
        int d2[6] = {cnt[0], cnt[1], cnt[2], cnt[1], cnt[2], cnt[2]};
        for (int g = 0; g < 6; g++) {
          b->gam_off[q * 6 + g] = off;
          b->gam_n1[q * 6 + g] = d1[g];
          b->gam_n2[q * 6 + g] = d2[g];
          off += (long)d1[g] * d2[g];
          neq += sq[g] ? (long)d1[g] * (d1[g] + 1) / 2 : (long)d1[g] * d2[g];
        }
      }
  b->nfull = off;
  b->neq = neq;

  // orbits sharing (l, j, tz): jbas%states (basic_IMSRG.f90:302-340)
  std::vector<int> ljt_start(N), ljt_count(N), ljt_list;
  for (int a = 0; a < N; a++) {
    ljt_start[a] = (int)ljt_list.size();
    for (int i = 0; i < N; i++)
      if (b->jj[i] == b->jj[a] && b->ll[i] == b->ll[a] && b->itzp[i] == b->itzp[a]) ljt_list.push_back(i);
    ljt_count[a] = (int)ljt_list.size() - ljt_start[a];
  }
  std::vector<int> ph_pairs;
  for (int a = 0; a < P; a++)
    for (int i = 0; i < A; i++) {
      int ak = b->parts[a], ik = b->holes[i];
      if (b->jj[ak] == b->jj[ik] && b->ll[ak] == b->ll[ik] && b->itzp[ak] == b->itzp[ik]) {
        ph_pairs.push_back(a);
        ph_pairs.push_back(i);
      }
    }

  // cross-coupled layout (allocate_CCMAT, cross_coupled.f90:110-175)
  b->ccblocks = (jtm + 1) * 4;
  b->cc_rlen.assign(b->ccblocks, 0);
  b->cc_nph.assign(b->ccblocks, 0);
  b->cc_J2.assign(b->ccblocks, 0);
  b->cc_off.assign(b->ccblocks, 0);
  b->wcc_off.assign(b->ccblocks, 0);
  std::vector<int> cc_row((size_t)b->ccblocks * N * N, -1);
  std::vector<int> cc_rowpair, cc_rowstart(b->ccblocks), cc_colpair, cc_colstart(b->ccblocks);
  long coff = 0, woff = 0;
  for (int q1 = 0; q1 < b->ccblocks; q1++) {
    int JC = (q1 % (jtm + 1)) * 2;
    int PAR = q1 / (2 * jtm + 2);
    int TZ = (q1 % (2 * jtm + 2)) / (jtm + 1);
    cc_rowstart[q1] = (int)cc_rowpair.size();
    cc_colstart[q1] = (int)cc_colpair.size();
    int r = 0, nb = 0;
    for (int i = 0; i < N; i++)
      for (int j = 0; j < N; j++) {
        if (!tri(b->jj[i], b->jj[j], JC)) continue;
        if ((b->ll[i] + b->ll[j]) % 2 != PAR) continue;
        if (std::abs(b->itzp[i] - b->itzp[j]) / 2 != TZ) continue;
        cc_row[((size_t)q1 * N + i) * N + j] = r++;
        cc_rowpair.push_back(i * 65536 + j);
        if (b->con[i] == 0 && b->con[j] == 1) {
          cc_colpair.push_back(i * 65536 + j);
          nb++;
        }
      }
    b->cc_rlen[q1] = r;
    b->cc_nph[q1] = nb;
    b->cc_J2[q1] = JC;
    b->cc_off[q1] = coff;
    b->wcc_off[q1] = woff;
    coff += (long)r * nb;
    woff += (long)r * r;
  }
  b->cc_total = coff;
  b->wcc_total = woff;

  // 6j table: [j1h][j2h][j4h][j5h][J3][J6] for {j1 j2 J3; j4 j5 J6}
  SixJ sj;
  std::vector<double> six((size_t)nj * nj * nj * nj * nJ * nJ, 0.0);
  for (int a = 0; a < nj; a++)
    for (int c = 0; c < nj; c++)
      for (int d = 0; d < nj; d++)
        for (int e = 0; e < nj; e++)
          for (int J3 = 0; J3 < nJ; J3++)
            for (int J6 = 0; J6 < nJ; J6++)
              six[((((size_t)a * nj + c) * nj + d) * nj + e) * nJ * nJ + J3 * nJ + J6] =
                  sj(2 * a + 1, 2 * c + 1, 2 * J3, 2 * d + 1, 2 * e + 1, 2 * J6);

  // GEMM problems of 222_pp_hh per block, then the WCC products
  ProbBuilder pb;
  for (int qb = 0; qb < b->nblocks; qb++) {
    int np = b->npp[qb], nb = b->nph[qb], nh = b->nhh[qb];
    auto G = [&](int g) { return b->gam_off[qb * 6 + g - 1]; };
    // W1_pppp = L_pppp R_pppp
    pb.add(np, np, np, SRC_W1, G(1), np, {term(SRC_L, G(1), np, 0, SRC_R, G(1), np, 0, 1.0)});
    // W2_hhhh = L_hhhh R_hhhh
    pb.add(nh, nh, nh, SRC_W2, G(5), nh, {term(SRC_L, G(5), nh, 0, SRC_R, G(5), nh, 0, 1.0)});
    // W1_hhhh = herm_L L_pphh^T R_pphh
    pb.add(nh, nh, np, SRC_W1, G(5), nh, {term(SRC_L, G(3), np, 1, SRC_R, G(3), np, 0, 1.0, 1, 0)});
    // W2_pppp = herm_R L_pphh R_pphh^T
    pb.add(np, np, nh, SRC_W2, G(1), np, {term(SRC_L, G(3), np, 0, SRC_R, G(3), np, 1, 1.0, 0, 1)});
    // W1_pphh = L_pppp R_pphh - R_pppp L_pphh
    pb.add(np, nh, np, SRC_W1, G(3), np,
           {term(SRC_R, G(1), np, 0, SRC_L, G(3), np, 0, -1.0), term(SRC_L, G(1), np, 0, SRC_R, G(3), np, 0, 1.0)});
    // W2_pphh = L_pphh R_hhhh - R_pphh L_hhhh
    pb.add(np, nh, nh, SRC_W2, G(3), np,
           {term(SRC_R, G(3), np, 0, SRC_L, G(5), nh, 0, -1.0), term(SRC_L, G(3), np, 0, SRC_R, G(5), nh, 0, 1.0)});
    // W2_phph = herm_R L_phhh R_phhh^T
    pb.add(nb, nb, nh, SRC_W2, G(4), nb, {term(SRC_L, G(6), nb, 0, SRC_R, G(6), nb, 1, 1.0, 0, 1)});
    // W1_phph = herm_L L_ppph^T R_ppph
    pb.add(nb, nb, np, SRC_W1, G(4), nb, {term(SRC_L, G(2), np, 1, SRC_R, G(2), np, 0, 1.0, 1, 0)});
    // W2_phhh = L_phhh R_hhhh - R_phhh L_hhhh
    pb.add(nb, nh, nh, SRC_W2, G(6), nb,
           {term(SRC_R, G(6), nb, 0, SRC_L, G(5), nh, 0, -1.0), term(SRC_L, G(6), nb, 0, SRC_R, G(5), nh, 0, 1.0)});
    // W1_ppph = L_pppp R_ppph - R_pppp L_ppph
    pb.add(np, nb, np, SRC_W1, G(2), np,
           {term(SRC_R, G(1), np, 0, SRC_L, G(2), np, 0, -1.0), term(SRC_L, G(1), np, 0, SRC_R, G(2), np, 0, 1.0)});
    // W1_phhh = -herm_R R_ppph^T L_pphh + herm_L L_ppph^T R_pphh
    pb.add(nb, nh, np, SRC_W1, G(6), nb,
           {term(SRC_R, G(2), np, 1, SRC_L, G(3), np, 0, -1.0, 0, 1),
            term(SRC_L, G(2), np, 1, SRC_R, G(3), np, 0, 1.0, 1, 0)});
    // W2_ppph = herm_R L_pphh R_phhh^T - herm_L R_pphh L_phhh^T
    pb.add(np, nb, nh, SRC_W2, G(2), np,
           {term(SRC_R, G(3), np, 0, SRC_L, G(6), nb, 1, -1.0, 1, 0),
            term(SRC_L, G(3), np, 0, SRC_R, G(6), nb, 1, 1.0, 0, 1)});
  }
  for (int q1 = 0; q1 < b->ccblocks; q1++) {
    int r = b->cc_rlen[q1], nb = b->cc_nph[q1];
    pb.add(r, r, nb, SRC_WCC, b->wcc_off[q1], r,
           {term(SRC_LCC, b->cc_off[q1], r, 0, SRC_RCC, b->cc_off[q1], r, 1, 1.0)});
  }
  // FP64 tiles: 64 x 64, or 256 x 8 for the problems whose output has at
  // most eight columns (the hole-pair-wide ladder products), which a 64-wide
  // tile would mostly pad
  int tiles = 0;
  for (GemmProb &p : pb.probs) {
    p.shape = p.N <= 8 ? 1 : 0;
    if (p.shape == 1) {
      p.tiles_m = (p.M + 255) / 256;
      p.tiles = p.tiles_m;
    } else {
      p.tiles_m = (p.M + 63) / 64;
      p.tiles = p.tiles_m * ((p.N + 63) / 64);
    }
    p.tile0 = tiles;
    tiles += p.tiles;
  }
  b->probs = pb.probs;
  b->nprobs = (int)pb.probs.size();
  b->ntiles = tiles;

  // norm chunks (mat_frob_norm weights: fph and non-square gam count twice)
  std::vector<NormChunk> chunks;
  auto add_seg = [&](long start, long len, int w) {
    for (long s = 0; s < len; s += 4096) {
      NormChunk c{start + s, (int)std::min<long>(4096, len - s), w};
      chunks.push_back(c);
    }
  };
  add_seg(b->off_fhh, (long)A * A, 1);
  add_seg(b->off_fph, (long)P * A, 2);
  add_seg(b->off_fpp, (long)P * P, 1);
  for (int qb = 0; qb < b->nblocks; qb++)
    for (int g = 0; g < 6; g++)
      add_seg(b->gam_off[qb * 6 + g], (long)b->gam_n1[qb * 6 + g] * b->gam_n2[qb * 6 + g], sq[g] ? 1 : 2);
  b->nchunks = (int)chunks.size();

  // packed (vectorize) map
  std::vector<long> psrc, pmir;
  psrc.reserve(neq);
  pmir.reserve(neq);
  psrc.push_back(0);
  pmir.push_back(-1);
  for (long k = 0; k < (long)A * A; k++) { psrc.push_back(b->off_fhh + k); pmir.push_back(-1); }
  for (long k = 0; k < (long)P * P; k++) { psrc.push_back(b->off_fpp + k); pmir.push_back(-1); }
  for (long k = 0; k < (long)P * A; k++) { psrc.push_back(b->off_fph + k); pmir.push_back(-1); }
  for (int qb = 0; qb < b->nblocks; qb++)
    for (int g = 0; g < 6; g++) {
      int n1 = b->gam_n1[qb * 6 + g], n2 = b->gam_n2[qb * 6 + g];
      long o = b->gam_off[qb * 6 + g];
      for (int i = 0; i < n2; i++)
        for (int j = sq[g] ? i : 0; j < n1; j++) {
          psrc.push_back(o + j + (long)i * n1);
          pmir.push_back(sq[g] ? o + i + (long)j * n1 : -1);
        }
    }
  if ((long)psrc.size() != neq) return IMSRG_ERR_INVALID;

  // --- device copies
  cudaError_t ce = cudaGetDevice(&b->device);
  if (ce != cudaSuccess) return cuda_status(ce);
  IMSRG_CUDA_TRY(cudaDeviceGetAttribute(&b->num_sms, cudaDevAttrMultiProcessorCount, b->device));
  IMSRG_CUDA_TRY(cudaStreamCreateWithFlags(&b->own_stream, cudaStreamNonBlocking));
  b->stream = b->own_stream;
  IMSRG_CUDA_TRY(cudaStreamCreateWithFlags(&b->side, cudaStreamNonBlocking));
  IMSRG_CUDA_TRY(cudaStreamCreateWithFlags(&b->side2, cudaStreamNonBlocking));
  IMSRG_CUDA_TRY(cudaStreamCreateWithFlags(&b->side3, cudaStreamNonBlocking));
  IMSRG_CUDA_TRY(cudaStreamCreateWithFlags(&b->side4, cudaStreamNonBlocking));
  IMSRG_CUDA_TRY(cudaEventCreateWithFlags(&b->ev_join3, cudaEventDisableTiming));
  IMSRG_CUDA_TRY(cudaEventCreateWithFlags(&b->ev_pre, cudaEventDisableTiming));
  IMSRG_CUDA_TRY(cudaEventCreateWithFlags(&b->ev_rdev, cudaEventDisableTiming));
  IMSRG_CUDA_TRY(cudaEventCreateWithFlags(&b->ev_join2, cudaEventDisableTiming));
  IMSRG_CUDA_TRY(cudaEventCreateWithFlags(&b->ev_hostL, cudaEventDisableTiming));
  for (int k = 0; k < 2; k++) {
    IMSRG_CUDA_TRY(cudaEventCreateWithFlags(&b->ev_fork[k], cudaEventDisableTiming));
    IMSRG_CUDA_TRY(cudaEventCreateWithFlags(&b->ev_join[k], cudaEventDisableTiming));
  }
  IMSRG_CUDA_TRY(cudaEventCreateWithFlags(&b->ev_hostR, cudaEventDisableTiming));
  IMSRG_CUDA_TRY(cudaEventCreateWithFlags(&b->ev_outj, cudaEventDisableTiming));
  for (cudaEvent_t &ev : b->ev_out) IMSRG_CUDA_TRY(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
  DevTables &T = b->T;
  T.norb = N;
  T.A = A;
  T.P = P;
  T.nblocks = b->nblocks;
  T.jtm = jtm;
  T.nJ = nJ;
  T.nj = nj;
  T.ccblocks = b->ccblocks;
  T.off_fhh = b->off_fhh;
  T.off_fph = b->off_fph;
  T.off_fpp = b->off_fpp;
  T.nfull = b->nfull;
  T.cc_total = b->cc_total;
  T.wcc_total = b->wcc_total;
  std::vector<int4> orb(N);
  for (int i = 0; i < N; i++) orb[i] = make_int4(b->jj[i], b->ll[i], b->itzp[i], b->con[i]);
  std::vector<int> qn_flat, qn_start(b->nblocks * 3);
  for (int k = 0; k < b->nblocks * 3; k++) {
    qn_start[k] = (int)qn_flat.size();
    qn_flat.insert(qn_flat.end(), b->qn[k].begin(), b->qn[k].end());
  }
  IMSRG_TRY(dev_upload(b, orb, &T.orb));
  IMSRG_TRY(dev_upload(b, orbpos, &T.orbpos));
  IMSRG_TRY(dev_upload(b, pairrow, &T.pairrow));
  IMSRG_TRY(dev_upload(b, b->gam_off, &T.gam_off));
  IMSRG_TRY(dev_upload(b, b->gam_n1, &T.gam_n1));
  IMSRG_TRY(dev_upload(b, b->gam_n2, &T.gam_n2));
  IMSRG_TRY(dev_upload(b, blk_J2, &T.blk_J2));
  IMSRG_TRY(dev_upload(b, qn_flat, &T.qn));
  IMSRG_TRY(dev_upload(b, qn_start, &T.qn_start));
  IMSRG_TRY(dev_upload(b, six, &T.six));
  std::vector<double> six_w(six.size()), sqrt_j21(nJ), jp1(2 * nJ + 2);
  for (size_t k = 0; k < six.size(); k++) six_w[k] = (double)(2 * (k % nJ) + 1) * six[k];
  for (int J = 0; J < nJ; J++) sqrt_j21[J] = std::sqrt(2.0 * J + 1.0);
  for (int J2 = 0; J2 < 2 * nJ + 2; J2++) jp1[J2] = J2 + 1.0;
  IMSRG_TRY(dev_upload(b, six_w, &T.six_w));
  IMSRG_TRY(dev_upload(b, sqrt_j21, &T.sqrt_j21));
  IMSRG_TRY(dev_upload(b, jp1, &T.jp1));
  IMSRG_TRY(dev_upload(b, ljt_start, &T.ljt_start));
  IMSRG_TRY(dev_upload(b, ljt_count, &T.ljt_count));
  IMSRG_TRY(dev_upload(b, ljt_list, &T.ljt_list));
  IMSRG_TRY(dev_upload(b, cc_row, &T.cc_row));
  IMSRG_TRY(dev_upload(b, b->cc_off, &T.cc_off));
  IMSRG_TRY(dev_upload(b, b->wcc_off, &T.wcc_off));
  IMSRG_TRY(dev_upload(b, b->cc_rlen, &T.cc_rlen));
  IMSRG_TRY(dev_upload(b, b->cc_nph, &T.cc_nph));
  IMSRG_TRY(dev_upload(b, b->cc_J2, &T.cc_J2));
  IMSRG_TRY(dev_upload(b, cc_rowpair, &T.cc_rowpair));
  IMSRG_TRY(dev_upload(b, cc_rowstart, &T.cc_rowstart));
  IMSRG_TRY(dev_upload(b, cc_colpair, &T.cc_colpair));
  IMSRG_TRY(dev_upload(b, cc_colstart, &T.cc_colstart));
  IMSRG_TRY(dev_upload(b, ph_pairs, &T.ph_pairs));

  // --- element locations of v_elem (v_location) and f_elem (:1147-1177),
  // shared by every gather list below
  auto vloc = [&](int a, int bb, int c, int d, int J2) { return v_location(b, a, bb, c, d, J2); };
  // f_elem: flat index and whether the element is read transposed (a ph
  // element asked as hp takes the operator's herm)
  auto floc = [&](int a, int bb, int *trans) -> long {
    int ca = b->con[a], cb = b->con[bb];
    int pa = orbpos[a], pbp = orbpos[bb];
    *trans = 0;
    if (ca + cb == 0) return b->off_fpp + pa + (long)pbp * P;
    if (ca + cb == 2) return b->off_fhh + pa + (long)pbp * A;
    if (ca > cb) {
      *trans = 1;
      return b->off_fph + pbp + (long)pa * P;
    }
    return b->off_fph + pa + (long)pbp * P;
  };
  auto ccr = [&](int q1, int i, int j) { return cc_row[((size_t)q1 * N + i) * N + j]; };
  auto sixidx = [&](int j1, int j2, int J3, int j4, int j5, int J6) -> long {
    return ((((long)(j1 >> 1) * nj + (j2 >> 1)) * nj + (j4 >> 1)) * nj + (j5 >> 1)) * nJ * nJ + (J3 >> 1) * nJ +
           (J6 >> 1);
  };

  // --- two-body assembly: work order, gather lists and the recoupling inputs
  // shared by the elements of one orbit quadruple (see Asm2Head, PhTerm)
  {
    auto jpcount = [&](int lo, int hi) { return hi >= lo ? (hi - lo) / 2 + 1 : 0; };
    static const int c1tab[6] = {0, 0, 0, 1, 2, 1}, c2tab[6] = {0, 1, 2, 1, 2, 2};
    // elements of each (a, b, c, d, category), in increasing J (blocks run J-major)
    struct El {
      int e, em, J2, IX, JX;
    };
    std::map<unsigned long long, std::vector<El>> qmap;
    std::vector<unsigned long long> qorder;  // quadruples in first-seen order
    // sqrt(2) factors of every stored element (all of each array: a term may
    // read the lower triangle of a square one)
    std::vector<unsigned char> vsq(b->nfull, 0);
    for (int qb = 0; qb < b->nblocks; qb++)
      for (int g = 0; g < 6; g++) {
        const int n1 = b->gam_n1[qb * 6 + g], n2 = b->gam_n2[qb * 6 + g];
        const std::vector<int> &qr = b->qn[qb * 3 + c1tab[g]], &qc = b->qn[qb * 3 + c2tab[g]];
        for (int JX = 0; JX < n2; JX++)
          for (int IX = 0; IX < n1; IX++)
            vsq[b->gam_off[qb * 6 + g] + IX + (long)JX * n1] =
                (unsigned char)((qr[2 * IX] == qr[2 * IX + 1]) + (qc[2 * JX] == qc[2 * JX + 1]));
      }
    bool vsq_ok = true;  // every commutator_122 term's factor is its element's
    for (int qb = 0; qb < b->nblocks; qb++)
      for (int g = 0; g < 6; g++) {
        const int n1 = b->gam_n1[qb * 6 + g], n2 = b->gam_n2[qb * 6 + g];
        const std::vector<int> &qr = b->qn[qb * 3 + c1tab[g]], &qc = b->qn[qb * 3 + c2tab[g]];
        for (int JX = 0; JX < n2; JX++)
          for (int IX = 0; IX < n1; IX++) {
            if (sq[g] && IX > JX) continue;
            const unsigned long long key = ((((unsigned long long)qr[2 * IX] * 4096 + qr[2 * IX + 1]) * 4096 +
                                             qc[2 * JX]) * 4096 + qc[2 * JX + 1]) * 8 + g;
            auto it = qmap.find(key);
            if (it == qmap.end()) {
              it = qmap.emplace(key, std::vector<El>()).first;
              qorder.push_back(key);
            }
            El el{(int)(b->gam_off[qb * 6 + g] + IX + (long)JX * n1),
                  sq[g] ? (int)(b->gam_off[qb * 6 + g] + JX + (long)IX * n1) : -1, blk_J2[qb], IX, JX};
            it->second.push_back(el);
          }
      }
    std::vector<Asm2Head> heads;
    std::vector<PhTerm> zt;
    std::vector<unsigned long long> terms;
    std::vector<std::pair<long, int>> items;      // (signature, head)
    std::vector<std::pair<long, int>> items_out;  // (output range << 40 | signature, head)
    const long two0 = b->off_fpp + (long)P * P;  // first two-body index of the flat layout
    {  // output ranges: the first holds kOutFirst of the two-body part, the rest share the remainder
      const long span = b->nfull - two0;
      b->asm2_addr[0] = two0;
      for (int c = 1; c < kOutChunks; c++) {
        const double f = kOutFirst + (c - 1) * (1.0 - kOutFirst) / (kOutChunks - 1);
        b->asm2_addr[c] = two0 + (long)std::ceil(f * (double)span);
      }
      b->asm2_addr[kOutChunks] = b->nfull;
    }
    auto row16 = [](int r) -> unsigned long long { return r < 0 ? 0xFFFFull : (unsigned long long)r; };
    for (unsigned long long key : qorder) {
      const std::vector<El> &els = qmap[key];
      const int g = (int)(key & 7);
      const int l = (int)((key >> 3) & 4095), k = (int)((key >> 15) & 4095), j = (int)((key >> 27) & 4095),
                i = (int)((key >> 39) & 4095);
      const int ji = b->jj[i], jjv = b->jj[j], jk = b->jj[k], jl = b->jj[l];
      // commutator_222_ph recoupling inputs of both exchange channels (J independent)
      const int JTM = jtm;
      const int Tz1 = std::abs(b->itzp[i] - b->itzp[k]) / 2, PAR1 = (b->ll[i] + b->ll[k]) & 1;
      const int Tz2 = std::abs(b->itzp[i] - b->itzp[l]) / 2, PAR2 = (b->ll[i] + b->ll[l]) & 1;
      const bool valid = std::abs(b->itzp[l] - b->itzp[j]) == Tz1 * 2 && ((b->ll[l] + b->ll[j]) & 1) == PAR1 &&
                         std::abs(b->itzp[k] - b->itzp[j]) == Tz2 * 2 && ((b->ll[k] + b->ll[j]) & 1) == PAR2;
      const int nph = ((ji + jjv + jk + jl) >> 1) & 1;
      const int zs = (int)zt.size();
      const int jmin1 = std::max(std::abs(jjv - jl), std::abs(ji - jk)), jmax1 = std::min(jjv + jl, ji + jk);
      const int jmin2 = std::max(std::abs(ji - jl), std::abs(jjv - jk)), jmax2 = std::min(ji + jl, jjv + jk);
      int n_in = 0, n_out = 0;
      if (valid) {
        for (int JP = jmin1; JP <= jmax1; JP += 2, n_in++) {
          const int qx = JP / 2 + Tz1 * (JTM + 1) + 2 * PAR1 * (JTM + 1);
          zt.push_back({row16(ccr(qx, k, i)) | (row16(ccr(qx, j, l)) << 16) | (row16(ccr(qx, l, j)) << 32) |
                            (row16(ccr(qx, i, k)) << 48),
                        qx, nph});
        }
        for (int JP = jmin2; JP <= jmax2; JP += 2, n_out++) {
          const int qx = JP / 2 + Tz2 * (JTM + 1) + 2 * PAR2 * (JTM + 1);
          zt.push_back({row16(ccr(qx, l, i)) | (row16(ccr(qx, j, k)) << 16) | (row16(ccr(qx, k, j)) << 32) |
                            (row16(ccr(qx, i, l)) << 48),
                        qx, nph});
        }
      }
      const int nd = (i == j) + (k == l);
      for (const El &el : els) {
        const int J2 = el.J2;
        Asm2Head h{};
        h.e = el.e;
        h.em = el.em;
        h.J2 = J2;
        h.start = (int)terms.size();
        h.zs = zs;
        if (valid) {
          h.six1 = (int)sixidx(ji, jjv, J2, jl, jk, jmin1);
          h.six2 = (int)sixidx(ji, jjv, J2, jk, jl, jmin2);
        }
        // commutator_122: one-body insertions on the four legs
        auto add122 = [&](int leg_sign, int fa, int fb, const HLoc &v) {
          if (v.idx < 0) return;
          if (v.nsq != vsq[v.idx]) vsq_ok = false;
          int ftr;
          long fi = floc(fa, fb, &ftr);
          terms.push_back((unsigned long long)v.idx | ((unsigned long long)fi << 28) |
                          ((unsigned long long)(leg_sign ^ v.neg) << 48) | ((unsigned long long)v.nsq << 49) |
                          ((unsigned long long)v.trans << 51) | ((unsigned long long)ftr << 52));
        };
        for (int t = 0; t < ljt_count[i]; t++) {
          const int x = ljt_list[ljt_start[i] + t];
          add122(0, i, x, vloc(x, j, k, l, J2));
        }
        for (int t = 0; t < ljt_count[j]; t++) {
          const int x = ljt_list[ljt_start[j] + t];
          add122(0, j, x, vloc(i, x, k, l, J2));
        }
        for (int t = 0; t < ljt_count[k]; t++) {
          const int x = ljt_list[ljt_start[k] + t];
          add122(1, x, k, vloc(i, j, x, l, J2));
        }
        for (int t = 0; t < ljt_count[l]; t++) {
          const int x = ljt_list[ljt_start[l] + t];
          add122(1, x, l, vloc(i, j, k, x, J2));
        }
        const int n122 = (int)terms.size() - h.start;
        if (n122 > 31 || n_in > 31 || n_out > 31) return IMSRG_ERR_TOO_LARGE;
        const int n2par = (((jl + jk + J2) >> 1) + 1) & 1;
        h.meta = (unsigned)n122 | ((unsigned)n_in << 5) | ((unsigned)n_out << 10) | ((unsigned)valid << 15) |
                 ((unsigned)n2par << 16) | ((unsigned)nd << 18) | ((unsigned)(sq[g] && el.IX == el.JX) << 20) |
                 ((unsigned)sq[g] << 21) | ((unsigned)(g == 2) << 22);
        // warps run elements of one loop-trip signature; in the order by
        // output range, within the range of the element's lower write
        const long lo = el.em >= 0 ? std::min(el.e, el.em) : el.e;
        long chunk = 0;
        while (chunk + 1 < kOutChunks && lo >= b->asm2_addr[chunk + 1]) chunk++;
        const long sig = (((long)n_in * 32 + n_out) * 32 + n122) * 2 + (valid ? 1 : 0);
        items.push_back({sig, (int)heads.size()});
        items_out.push_back({chunk << 40 | sig, (int)heads.size()});
        heads.push_back(h);
      }
    }
    if (!vsq_ok) return IMSRG_ERR_INVALID;
    b->off_2b = two0;
    if (b->nfull >= (1L << 28) || b->off_fpp + (long)P * P >= (1L << 20)) return IMSRG_ERR_TOO_LARGE;
    for (int q1 = 0; q1 < b->ccblocks; q1++)
      if (b->cc_rlen[q1] >= 0xFFFF) return IMSRG_ERR_TOO_LARGE;
    auto by_key = [](const std::pair<long, int> &x, const std::pair<long, int> &y) { return x.first < y.first; };
    std::stable_sort(items.begin(), items.end(), by_key);
    std::stable_sort(items_out.begin(), items_out.end(), by_key);
    std::vector<Asm2Head> ordered(heads.size()), ordered_out(heads.size());
    for (size_t t = 0; t < items.size(); t++) {
      ordered[t] = heads[items[t].second];
      ordered_out[t] = heads[items_out[t].second];
    }
    for (int c = 0; c <= kOutChunks; c++)
      b->asm2_el[c] = std::lower_bound(items_out.begin(), items_out.end(), (long)c << 40,
                                       [](const std::pair<long, int> &x, long key) { return x.first < key; }) -
                      items_out.begin();
    T.n_asm2 = (int)ordered.size();
    T.n_ph = (int)zt.size();
    {  // the commutator_122 sums by term count, 32 elements to a warp (see DevTables::pre_warp)
      std::vector<std::vector<int>> by_n(32);
      for (size_t h = 0; h < heads.size(); h++) by_n[heads[h].meta & 31].push_back((int)h);
      std::vector<Asm2PreWarp> pw;
      std::vector<unsigned> pe;
      std::vector<unsigned long long> pt;
      for (int n = 0; n < 32; n++)
        for (size_t g0 = 0; g0 < by_n[n].size(); g0 += 32) {
          Asm2PreWarp w{(long long)pt.size(), n, 0};
          pw.push_back(w);
          pt.resize(pt.size() + (size_t)32 * n, 0ull);
          for (int l = 0; l < 32; l++) {
            if (g0 + l >= by_n[n].size()) {
              pe.push_back(0xFFFFFFFFu);
              continue;
            }
            const Asm2Head &h = heads[by_n[n][g0 + l]];
            const unsigned nd = (h.meta >> 18) & 3, diag = (h.meta >> 20) & 1;
            pe.push_back((unsigned)h.e | nd << 28 | diag << 30);
            for (int k = 0; k < n; k++) pt[(size_t)w.base + (size_t)32 * k + l] = terms[(size_t)h.start + k];
          }
        }
      T.n_pre_warps = (int)pw.size();
      IMSRG_TRY(dev_upload(b, pw, &T.pre_warp));
      IMSRG_TRY(dev_upload(b, pe, &T.pre_el));
      IMSRG_TRY(dev_upload(b, pt, &T.pre_terms));
    }
    IMSRG_TRY(dev_upload(b, ordered, &T.asm2_head));
    IMSRG_TRY(dev_upload(b, ordered_out, &T.asm2_head_out));
    IMSRG_TRY(dev_upload(b, terms, &T.asm2_terms));
    IMSRG_TRY(dev_upload(b, zt, &T.ph_terms));
    IMSRG_TRY(dev_upload(b, vsq, &T.vsq));

    std::vector<std::pair<long, int>> cit;
    T.ccf_packed = b->cc_total < (1L << 24) && b->ccblocks <= 128;
    for (int q1 = 0; q1 < b->ccblocks; q1++) {
      int rlen = b->cc_rlen[q1], nph = b->cc_nph[q1], JC = b->cc_J2[q1];
      const int *rows = cc_rowpair.data() + cc_rowstart[q1];
      const int *cols = cc_colpair.data() + cc_colstart[q1];
      for (int nb = 0; nb < nph; nb++)
        for (int r = 0; r < rlen; r++) {
          int a = rows[r] >> 16, bb = rows[r] & 0xffff, p = cols[nb] >> 16, h = cols[nb] & 0xffff;
          int n = 0;
          if ((b->ll[a] + b->ll[h]) % 2 == (b->ll[bb] + b->ll[p]) % 2 && b->itzp[a] + b->itzp[h] == b->itzp[bb] + b->itzp[p])
            n = jpcount(std::max(std::abs(b->jj[p] - b->jj[bb]), std::abs(b->jj[a] - b->jj[h])),
                        std::min(b->jj[p] + b->jj[bb], b->jj[a] + b->jj[h]));
          (void)JC;
          // the block id rides in bits 24-30 when it fits (the transform
          // then also reduces each block's largest exponent)
          const int packed = T.ccf_packed ? q1 << 24 : 0;
          cit.push_back({n, (int)(b->cc_off[q1] + r + (long)nb * rlen) | packed});
        }
    }
    // stable: within one term count the elements stay in block order, so the
    // lanes of a warp mostly share a block
    std::stable_sort(cit.begin(), cit.end(),
                     [](const std::pair<long, int> &x, const std::pair<long, int> &y) { return x.first < y.first; });
    std::vector<int> corder(cit.size());
    for (size_t t = 0; t < cit.size(); t++) corder[t] = cit[t].second;
    T.n_ccf = (int)corder.size();
    IMSRG_TRY(dev_upload(b, corder, &T.ccf_order));
  }

  // --- gather lists of the one-body assembly (commutators.f90:83-280, 435-578)
  {
    // location and prefactor (phase x sqrt(2)^nsq, rounded as the reference's
    // pre * sqrt(2) chain) of v_elem
    auto hloc = [&](int a, int bb, int c, int d, int J2, long *idx, double *pre, int *trans) {
      HLoc v = vloc(a, bb, c, d, J2);
      *idx = v.idx;
      if (v.idx < 0) return;
      double pr = v.neg ? -1.0 : 1.0;
      for (int k = 0; k < v.nsq; k++) pr = pr * 1.4142135623730951;
      *pre = pr;
      *trans = v.trans;
    };
    std::vector<OneBodyTerm> terms;
    long nel = (long)A * A + (long)P * A + (long)P * P;
    std::vector<int> ostart(nel), ocount(nel);
    auto same = [&](int x, int y) { return b->jj[x] == b->jj[y] && b->ll[x] == b->ll[y] && b->itzp[x] == b->itzp[y]; };
    for (long e = 0; e < nel; e++) {
      ostart[e] = (int)terms.size();
      int pk, qk;
      bool upper_only = true, with_pm = true;
      if (e < (long)A * A) {
        int p = (int)(e % A), q = (int)(e / A);
        pk = b->holes[p];
        qk = b->holes[q];
        if (p > q) upper_only = false;
      } else if (e < (long)A * A + (long)P * A) {
        long e2 = e - (long)A * A;
        pk = b->parts[e2 % P];
        qk = b->holes[e2 / P];
        with_pm = false;
      } else {
        long e3 = e - (long)A * A - (long)P * A;
        int p = (int)(e3 % P), q = (int)(e3 / P);
        pk = b->parts[p];
        qk = b->parts[q];
        if (p > q) upper_only = false;
      }
      if (!upper_only || !same(pk, qk)) {
        ocount[e] = 0;
        continue;
      }
      // commutator_121 inner sum (commutators.f90:117-150)
      int jq = b->jj[qk];
      for (size_t k = 0; k < ph_pairs.size() / 2; k++) {
        int a = ph_pairs[2 * k], i = ph_pairs[2 * k + 1];
        int ak = b->parts[a], ik = b->holes[i];
        int ji = b->jj[ik];
        int ph = a + i * P;
        for (int JT = std::abs(ji - jq); JT <= ji + jq; JT += 2) {
          long idx;
          double pr;
          int tr;
          hloc(ak, pk, ik, qk, JT, &idx, &pr, &tr);
          if (idx >= 0) terms.push_back({(int)idx, 0 | (tr << 2) | (ph << 8), (JT + 1.0) * pr});
          hloc(ik, pk, ak, qk, JT, &idx, &pr, &tr);
          if (idx >= 0) terms.push_back({(int)idx, 1 | (tr << 2) | (ph << 8), (JT + 1.0) * pr});
        }
      }
      // commutator_221 (commutators.f90:470-486)
      int ji = b->jj[pk];
      for (int c = 0; c < N; c++) {
        int jc = b->jj[c];
        int w2 = b->con[c] ? 0 : 1;
        for (int JT = std::abs(jc - ji); JT <= jc + ji; JT += 2) {
          long idx;
          double pr;
          int tr;
          hloc(c, pk, c, qk, JT, &idx, &pr, &tr);
          if (idx >= 0) terms.push_back({(int)idx, 2 | (w2 << 3), (JT + 1.0) * pr});
          if (with_pm) {
            hloc(c, qk, c, pk, JT, &idx, &pr, &tr);
            if (idx >= 0) terms.push_back({(int)idx, 3 | (w2 << 3), (JT + 1.0) * pr});
          }
        }
      }
      ocount[e] = (int)terms.size() - ostart[e];
    }
    IMSRG_TRY(dev_upload(b, terms, &T.obt));
    IMSRG_TRY(dev_upload(b, ostart, &T.obt_start));
    IMSRG_TRY(dev_upload(b, ocount, &T.obt_count));
    // work split of the one-body kernel: allowed upper-triangle elements
    // (longest gather list first) and all elements without a gather list
    std::vector<int> heavy, light;
    for (long e = 0; e < nel; e++) {
      int pk, qk, p = 0, q = 0;
      bool square = true;
      if (e < (long)A * A) {
        p = (int)(e % A);
        q = (int)(e / A);
        pk = b->holes[p];
        qk = b->holes[q];
      } else if (e < (long)A * A + (long)P * A) {
        long e2 = e - (long)A * A;
        pk = b->parts[e2 % P];
        qk = b->holes[e2 / P];
        square = false;
      } else {
        long e3 = e - (long)A * A - (long)P * A;
        p = (int)(e3 % P);
        q = (int)(e3 / P);
        pk = b->parts[p];
        qk = b->parts[q];
      }
      if (!same(pk, qk)) light.push_back((int)e);
      else if (!square || p <= q) heavy.push_back((int)e);
    }
    std::stable_sort(heavy.begin(), heavy.end(), [&](int x, int y) { return ocount[x] > ocount[y]; });
    T.n_asm1_heavy = (int)heavy.size();
    T.n_asm1_light = (int)light.size();
    IMSRG_TRY(dev_upload(b, heavy, &T.asm1_heavy));
    IMSRG_TRY(dev_upload(b, light, &T.asm1_light));

    // Pandya transform, cross_coupled.f90:1247-1291: CCX(r(a,b), nb(p,h)) =
    // (-1)^((jh+jb+J')/2) sqrt(2J'+1) sum_J (-1)^J (2J+1) {jp jh J'; ja jb J} V^J_{hapb}
    std::vector<int> cstart(b->cc_total + 1), cidx;
    std::vector<double> ccoef;
    for (int q1 = 0; q1 < b->ccblocks; q1++) {
      int rlen = b->cc_rlen[q1], nph = b->cc_nph[q1], JC = b->cc_J2[q1];
      const int *rows = cc_rowpair.data() + cc_rowstart[q1];
      const int *cols = cc_colpair.data() + cc_colstart[q1];
      for (int nb = 0; nb < nph; nb++)
        for (int r = 0; r < rlen; r++) {
          long e = b->cc_off[q1] + r + (long)nb * rlen;
          cstart[e] = (int)cidx.size();
          int a = rows[r] >> 16, bb = rows[r] & 0xffff, p = cols[nb] >> 16, h = cols[nb] & 0xffff;
          if (!((b->ll[a] + b->ll[h]) % 2 == (b->ll[bb] + b->ll[p]) % 2 &&
                b->itzp[a] + b->itzp[h] == b->itzp[bb] + b->itzp[p]))
            continue;
          int jp = b->jj[p], jh = b->jj[h], ja = b->jj[a], jb = b->jj[bb];
          double outer = (((jh + jb + JC) / 2) % 2 ? -1.0 : 1.0) * std::sqrt(JC + 1.0);
          for (int JT = std::max(std::abs(jp - jb), std::abs(ja - jh)); JT <= std::min(jp + jb, ja + jh); JT += 2) {
            long idx;
            double pr;
            int tr;
            hloc(h, a, p, bb, JT, &idx, &pr, &tr);
            if (idx < 0) continue;
            double s6 = six[((((size_t)(jp >> 1) * nj + (jh >> 1)) * nj + (ja >> 1)) * nj + (jb >> 1)) * nJ * nJ +
                            (JC >> 1) * nJ + (JT >> 1)];
            double w = ((JT / 2) % 2 ? -1.0 : 1.0) * (JT + 1) * s6;
            cidx.push_back((int)idx | (tr ? (int)0x80000000u : 0));
            ccoef.push_back(w * outer * pr);
          }
        }
    }
    cstart[b->cc_total] = (int)cidx.size();
    IMSRG_TRY(dev_upload(b, cstart, &T.cct_start));
    IMSRG_TRY(dev_upload(b, cidx, &T.cct_idx));
    IMSRG_TRY(dev_upload(b, ccoef, &T.cct_coef));
  }
  IMSRG_TRY(dev_upload(b, b->holes, &T.hole_orb));
  IMSRG_TRY(dev_upload(b, b->parts, &T.part_orb));
  T.n_ph_pairs = (int)ph_pairs.size() / 2;
  const GemmProb *dp = nullptr;
  IMSRG_TRY(dev_upload(b, b->probs, &dp));
  b->d_probs = (GemmProb *)dp;
  const NormChunk *dc = nullptr;
  IMSRG_TRY(dev_upload(b, chunks, &dc));
  b->d_chunks = (NormChunk *)dc;
  const long *d1 = nullptr, *d2 = nullptr;
  IMSRG_TRY(dev_upload(b, psrc, &d1));
  IMSRG_TRY(dev_upload(b, pmir, &d2));
  b->d_pack_src = (long *)d1;
  b->d_pack_mirror = (long *)d2;

  void *p = nullptr;
  IMSRG_TRY(dev_alloc(b, b->nfull * sizeof(double), &p));
  b->w1 = (double *)p;
  IMSRG_TRY(dev_alloc(b, b->nfull * sizeof(double), &p));
  b->w2 = (double *)p;
  IMSRG_TRY(dev_alloc(b, b->cc_total * sizeof(double), &p));
  b->lcc = (double *)p;
  IMSRG_TRY(dev_alloc(b, b->cc_total * sizeof(double), &p));
  b->rcc = (double *)p;
  IMSRG_TRY(dev_alloc(b, b->wcc_total * sizeof(double), &p));
  b->wcc = (double *)p;
  IMSRG_TRY(dev_alloc(b, (size_t)T.n_ph * sizeof(double), &p));
  b->zph = (double *)p;
  IMSRG_TRY(dev_alloc(b, (size_t)2 * N * N * sizeof(double), &p));  // monopoles of H and of a tangent dH
  b->mono = (double *)p;
  IMSRG_TRY(dev_alloc(b, 64 * sizeof(double), &p));
  b->scal = (double *)p;
  b->partials_len = std::max(std::max(b->nchunks, b->nblocks), asm2_ctas(b)) + 64;
  IMSRG_TRY(dev_alloc(b, b->partials_len * sizeof(double), &p));
  b->partials = (double *)p;
  IMSRG_TRY(dev_alloc(b, std::max(b->nfull, b->neq) * sizeof(double), &p));
  b->d_stage = (double *)p;
  IMSRG_CUDA_TRY(cudaMallocHost(&b->h_scal, 64 * sizeof(double)));
  IMSRG_CUDA_TRY(cudaMallocHost(&b->h_stage, std::max(b->nfull, b->neq) * sizeof(double)));
  IMSRG_CUDA_TRY(cudaDeviceSynchronize());
  return IMSRG_OK;
}

void free_basis_device(imsrg_basis *b) {
  if (b->stream) cudaStreamSynchronize(b->stream);
  profile_free(b);
  flow_graph_free(b);
  adjoint_free(b);
  for (imsrg_basis::CommGraph &g : b->comm_graphs) cudaGraphExecDestroy(g.exec);
  b->comm_graphs.clear();
  ozaki_free(b);
  for (void *p : b->dev_allocs) cudaFree(p);
  b->dev_allocs.clear();
  if (b->h_scal) cudaFreeHost(b->h_scal);
  if (b->h_stage) cudaFreeHost(b->h_stage);
  b->h_scal = b->h_stage = nullptr;
  if (b->own_stream) cudaStreamDestroy(b->own_stream);
  b->stream = b->own_stream = nullptr;
  if (b->side) cudaStreamDestroy(b->side);
  if (b->side2) cudaStreamDestroy(b->side2);
  if (b->side3) cudaStreamDestroy(b->side3);
  if (b->side4) cudaStreamDestroy(b->side4);
  b->side = b->side2 = b->side3 = b->side4 = nullptr;
  if (b->ev_join3) cudaEventDestroy(b->ev_join3);
  if (b->ev_pre) cudaEventDestroy(b->ev_pre);
  if (b->ev_rdev) cudaEventDestroy(b->ev_rdev);
  b->ev_join3 = b->ev_pre = b->ev_rdev = nullptr;
  if (b->ev_join2) cudaEventDestroy(b->ev_join2);
  if (b->ev_hostL) cudaEventDestroy(b->ev_hostL);
  if (b->ev_hostR) cudaEventDestroy(b->ev_hostR);
  if (b->ev_outj) cudaEventDestroy(b->ev_outj);
  b->ev_join2 = b->ev_hostL = b->ev_hostR = b->ev_outj = nullptr;
  for (cudaEvent_t &ev : b->ev_out) {
    if (ev) cudaEventDestroy(ev);
    ev = nullptr;
  }
  for (int k = 0; k < 2; k++) {
    if (b->ev_fork[k]) cudaEventDestroy(b->ev_fork[k]);
    if (b->ev_join[k]) cudaEventDestroy(b->ev_join[k]);
    b->ev_fork[k] = b->ev_join[k] = nullptr;
  }
}

}  // namespace imsrg
