// setup.cu -- the steps before the flow (main_IMSRG.f90:127-157):
//   * read_interaction (interaction_IO.f90:8-107): the ASCII two-body file of
//     VRenormalize with its centre-of-mass and Lawson terms, which need the
//     r1.r2 and p1.p2 HO matrix elements (basic_IMSRG.f90:4310-4530);
//   * calculate_h0_harm_osc (basic_IMSRG.f90:2049-2147): the HO one-body part;
//   * calc_HF (HF_mod.f90:14-106) without a three-body force, on the GPU:
//     density matrices (:346-373), the Hartree-Fock potential (gamma_matrix,
//     :169-232) as one gather over a host-built term list, the Fock matrices
//     of the (l, j, tz) blocks diagonalised by cyclic Jacobi (the reference
//     calls LAPACK dsyev, basic_IMSRG.f90:2163-2180), the one-body
//     transformation (:408-491) and the two-body one (:494-619).  The
//     reference's four products C^T V C, C^T V Crev, Crev^T V C, Crev^T V
//     Crev combined as V1 - s (V2 + V3) + V4 (s = (-1)^J) equal E^T V E with
//     E = C - s Crev (s^2 = 1), which is two GEMMs per block instead of eight.
// File parsing and the one-body HO matrix are host work (I/O and a few
// thousand numbers); everything that scales with the two-body space runs on
// the device.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "device.cuh"

namespace imsrg {

namespace {

int op_ok(const imsrg_op *op) { return (op && op->b && op->d) ? IMSRG_OK : IMSRG_ERR_INVALID; }

// (-1)^n for any integer n
inline double phase(int n) { return (n & 1) ? -1.0 : 1.0; }

// <a||r||c> and <a||p||c> of HO orbits in oscillator units (reduced_r,
// reduced_p of basic_IMSRG.f90); only l differing by one and n by at most
// one contribute
double reduced_rp(const imsrg_basis *b, int a, int c, bool p) {
  const int la = b->ll[a], lc = b->ll[c], na = b->nn[a], nc = b->nn[c];
  double c1 = 0.0, p1 = 0.0;
  if (la == lc + 1) {
    c1 = std::sqrt(lc + 1.0);
    if (na == nc) p1 = (p ? -1.0 : 1.0) * std::sqrt(nc + lc + 1.5);
    else if (na == nc - 1) p1 = -std::sqrt(nc * 1.0);
  } else if (la == lc - 1) {
    c1 = -std::sqrt(1.0 * lc);
    if (na == nc) p1 = std::sqrt(nc + lc + 0.5);
    else if (na == nc + 1) p1 = (p ? 1.0 : -1.0) * std::sqrt(nc + 1.0);
  }
  return p1 * c1;
}

// the spin-orbit recoupled single-particle factor of r1_r2 / p1_p2
double jfac(const imsrg_basis *b, int x, int y, bool p) {
  if (b->itzp[x] != b->itzp[y]) return 0.0;
  const double red = reduced_rp(b, x, y, p);
  if (red == 0.0) return 0.0;
  const int jx = b->jj[x], jy = b->jj[y], lx = b->ll[x], ly = b->ll[y];
  return std::sqrt((jx + 1.0) * (jy + 1.0)) * phase((3 + 2 * lx + jy) / 2) * sixj(jx, 2, jy, 2 * ly, 1, 2 * lx) * red;
}

// r1.r2 (times b^2) or p1.p2 (over b^2) between normalised kets |a b; J>,
// |c d; J> (r1_r2 / p1_p2, basic_IMSRG.f90:4310-4420)
double r1r2_p1p2(const imsrg_basis *b, int a, int bb, int c, int d, int J2, bool p) {
  const int ja = b->jj[a], jb = b->jj[bb], jc = b->jj[c], jd = b->jj[d];
  const double j_ac = jfac(b, a, c, p), j_ad = jfac(b, a, d, p), j_bc = jfac(b, bb, c, p), j_bd = jfac(b, bb, d, p);
  const int s1 = p ? (jb - jc - J2) / 2 : (jb + jc - J2) / 2;
  const int s2 = p ? (jb - jd - J2) / 2 : (jb + jd - J2) / 2;
  const double v = phase(s1) * sixj(ja, jb, J2, jd, jc, 2) * j_ac * j_bd -
                   phase((jc + jd - J2) / 2) * phase(s2) * sixj(ja, jb, J2, jc, jd, 2) * j_ad * j_bc;
  return v / std::sqrt((1.0 + (a == bb)) * (1.0 + (c == d)));
}

// ---------------------------------------------------------------------------
// Hartree-Fock device work
// ---------------------------------------------------------------------------
constexpr int HF_MAXN = 16;  // largest (l, j, tz) block (emax <= 30)

struct SpBlock {
  int n, off, j2, st0;  // states, offset of its n x n matrices, 2j, first entry in the state list
};

// rho = (2j + 1) Dx Dx^T with Dx the eigenvectors of hole states
// (density_matrix, HF_mod.f90:346-373); one thread per matrix element
__global__ void k_hf_density(const SpBlock *blk, int nblk, const int *states, const int *con, const double *D,
                             double *rho) {
  const int q = blockIdx.x;
  if (q >= nblk) return;
  const SpBlock B = blk[q];
  for (int e = threadIdx.x; e < B.n * B.n; e += blockDim.x) {
    const int a = e % B.n, c = e / B.n;
    double s = 0.0;
    for (int i = 0; i < B.n; i++)
      if (con[states[B.st0 + i]]) s = fma(D[B.off + a + i * B.n], D[B.off + c + i * B.n], s);
    rho[B.off + e] = s * (B.j2 + 1.0);
  }
}

// gamma_matrix (HF_mod.f90:169-232): each Fock element (q, i, j) sums
// rho(h, g) v_elem(...) (J + 1) / (j_rho + 1) / (j + 1) over its terms; one
// warp per element, fixed order
struct HfTerm {
  int rho;    // index into rho
  long v;     // flat index of the two-body element
  double c;   // phase, sqrt(2) factors and the angular weights
};

__global__ void k_hf_gamma(const int *elem_start, const int2 *elem_pos, int nelem, const HfTerm *terms,
                           const double *rho, const double *V, double *G) {
  const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (w >= nelem) return;
  double s = 0.0;
  for (int k = elem_start[w] + lane; k < elem_start[w + 1]; k += 32) {
    const HfTerm t = terms[k];
    s = fma(rho[t.rho] * t.c, V[t.v], s);
  }
  s = warp_sum(s);
  if (lane == 0) {
    const int2 p = elem_pos[w];  // (index of (i, j), index of (j, i))
    G[p.x] = s;
    G[p.y] = s;
  }
}

// F = T + G and its eigen-decomposition by cyclic Jacobi rotations (Golub and
// Van Loan, the symmetric Schur decomposition), eigenvalues ascending with
// their eigenvectors as the columns of D; one thread per block
__global__ void k_hf_diag(const SpBlock *blk, int nblk, const double *T, const double *G, double *D, double *eig,
                          int *eig_off) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nblk) return;
  const SpBlock B = blk[q];
  const int n = B.n;
  if (n == 0) return;
  double a[HF_MAXN][HF_MAXN], v[HF_MAXN][HF_MAXN];
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++) {
      a[i][j] = T[B.off + i + j * n] + G[B.off + i + j * n];
      v[i][j] = i == j ? 1.0 : 0.0;
    }
  for (int sweep = 0; sweep < 60; sweep++) {
    double off = 0.0, diag = 0.0;
    for (int i = 0; i < n; i++) {
      diag += a[i][i] * a[i][i];
      for (int j = i + 1; j < n; j++) off += a[i][j] * a[i][j];
    }
    if (off <= 1e-32 * diag || off == 0.0) break;
    for (int p = 0; p < n - 1; p++)
      for (int r = p + 1; r < n; r++) {
        if (a[p][r] == 0.0) continue;
        const double theta = (a[r][r] - a[p][p]) / (2.0 * a[p][r]);
        const double t = (theta >= 0.0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
        const double c = 1.0 / sqrt(t * t + 1.0), s = t * c;
        for (int k = 0; k < n; k++) {  // A <- J^T A J, V <- V J
          const double akp = a[k][p], akr = a[k][r];
          a[k][p] = c * akp - s * akr;
          a[k][r] = s * akp + c * akr;
        }
        for (int k = 0; k < n; k++) {
          const double apk = a[p][k], ark = a[r][k];
          a[p][k] = c * apk - s * ark;
          a[r][k] = s * apk + c * ark;
        }
        for (int k = 0; k < n; k++) {
          const double vkp = v[k][p], vkr = v[k][r];
          v[k][p] = c * vkp - s * vkr;
          v[k][r] = s * vkp + c * vkr;
        }
      }
  }
  int ord[HF_MAXN];
  for (int i = 0; i < n; i++) ord[i] = i;
  for (int i = 0; i < n; i++)  // selection sort, ascending (ties keep their order)
    for (int j = i + 1; j < n; j++)
      if (a[ord[j]][ord[j]] < a[ord[i]][ord[i]]) {
        const int t = ord[i];
        ord[i] = ord[j];
        ord[j] = t;
      }
  for (int i = 0; i < n; i++) {
    eig[eig_off[q] + i] = a[ord[i]][ord[i]];
    for (int k = 0; k < n; k++) D[B.off + k + i * n] = v[k][ord[i]];
  }
}

// the sign convention of calc_HF (:74-81): every eigenvector has a
// non-negative diagonal entry; then X' = D^T X D for X = F (= T + G), T, G
__global__ void k_hf_transform1(const SpBlock *blk, int nblk, double *D, double *T, double *G, double *F) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nblk) return;
  const SpBlock B = blk[q];
  const int n = B.n;
  if (n == 0) return;
  double *d = D + B.off;
  for (int i = 0; i < n; i++)
    if (d[i + i * n] < 0.0)
      for (int k = 0; k < n; k++) d[k + i * n] = -d[k + i * n];
  for (int m = 0; m < 3; m++) {
    double *X = m == 0 ? F : m == 1 ? T : G;
    double x[HF_MAXN][HF_MAXN], y[HF_MAXN][HF_MAXN];
    for (int i = 0; i < n; i++)
      for (int j = 0; j < n; j++)
        x[i][j] = m == 0 ? T[B.off + i + j * n] + G[B.off + i + j * n] : X[B.off + i + j * n];
    for (int i = 0; i < n; i++)  // y = X D
      for (int j = 0; j < n; j++) {
        double s = 0.0;
        for (int k = 0; k < n; k++) s = fma(x[i][k], d[k + j * n], s);
        y[i][j] = s;
      }
    for (int i = 0; i < n; i++)  // X' = D^T y
      for (int j = 0; j < n; j++) {
        double s = 0.0;
        for (int k = 0; k < n; k++) s = fma(d[k + i * n], y[k][j], s);
        X[B.off + i + j * n] = s;
      }
  }
}

// One two-body block of the transformation: rows/columns ordered hh, ph, pp
// pairs as transform_2b_to_HF assembles its square matrix.
struct HfBlock2 {
  int q, nh, nb, np, nt;
  long off;  // of its nt x nt matrices in the workspace
  int pair0; // first of its nt pairs in the pair list
  int sgn;   // (-1)^J
};

// Vfull from the six arrays (symmetric; transform_2b_to_HF :538-553) and
// E = C - s Crev (:561-585); one CTA per block
__global__ void k_hf_vfull(const HfBlock2 *blks, const long *gam_off, const int *gam_n1, const double *H,
                           const int2 *pairs, const double *Dsm, int norb, const int *jj, double *Vf, double *E) {
  const HfBlock2 B = blks[blockIdx.x];
  const int nt = B.nt, nh = B.nh, nb = B.nb;
  auto cat = [&](int r, int *local) {  // 5 = hh, 4 = ph, 0 = pp  (qn categories 2, 1, 0)
    if (r < nh) {
      *local = r;
      return 2;
    }
    if (r < nh + nb) {
      *local = r - nh;
      return 1;
    }
    *local = r - nh - nb;
    return 0;
  };
  // gam index of (row category, column category), and whether the stored
  // array is indexed (column, row)
  for (long e = threadIdx.x; e < (long)nt * nt; e += blockDim.x) {
    const int r = (int)(e % nt), c = (int)(e / nt);
    int lr, lc;
    const int cr = cat(r, &lr), cc = cat(c, &lc);
    // arrays: 0 pppp (pp,pp) 1 ppph (pp,ph) 2 pphh (pp,hh) 3 phph (ph,ph) 4 hhhh (hh,hh) 5 phhh (ph,hh)
    int g, i1 = lr, i2 = lc;
    const int lo = cr < cc ? cr : cc, hi = cr < cc ? cc : cr;
    if (lo == 0 && hi == 0) g = 0;
    else if (lo == 0 && hi == 1) g = 1;
    else if (lo == 0 && hi == 2) g = 2;
    else if (lo == 1 && hi == 1) g = 3;
    else if (lo == 2 && hi == 2) g = 4;
    else g = 5;
    if (cr > cc) {  // stored with the lower category as the row
      i1 = lc;
      i2 = lr;
    }
    const long sg = (long)B.q * 6 + g;
    Vf[B.off + e] = H[gam_off[sg] + i1 + (long)i2 * gam_n1[sg]];
    // E(JJ, II): JJ = r old pair (a, b), II = c new pair (i, j)
    const int2 pab = pairs[B.pair0 + r], pij = pairs[B.pair0 + c];
    const int a = pab.x, bq = pab.y, i = pij.x, j = pij.y;
    const double nrm = sqrt(1.0 + (a == bq)) / sqrt(1.0 + (i == j));
    const double cf = Dsm[a + (long)i * norb] * Dsm[bq + (long)j * norb] * nrm;
    const double cr2 = (a == bq) ? 0.0
                                 : Dsm[bq + (long)i * norb] * Dsm[a + (long)j * norb] *
                                       (((jj[a] + jj[bq]) / 2) & 1 ? -1.0 : 1.0) * nrm;
    E[B.off + e] = cf - B.sgn * cr2;
  }
}

// Y = op(A) B for the nt x nt matrices of every block (op(A) = A or A^T),
// 32 x 32 tiles of 256 threads, 4 outputs each
struct HfGemm {
  long a, bm, y;  // offsets in the workspace
  int nt, ta, tile0, tiles_1d;
};

__global__ void __launch_bounds__(256) k_hf_gemm(const HfGemm *probs, int nprobs, const double *W0, const double *W1,
                                                 double *Y) {
  __shared__ double As[32][33], Bs[32][33];
  const int tile = blockIdx.x;
  int lo = 0, hi = nprobs;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (probs[mid].tile0 <= tile) lo = mid + 1;
    else hi = mid;
  }
  const HfGemm P = probs[lo - 1];
  const int lt = tile - P.tile0, tm = lt % P.tiles_1d, tn = lt / P.tiles_1d, nt = P.nt;
  const double *A = W0 + P.a, *Bm = W1 + P.bm;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;  // 32 x 8
  double acc[4] = {0.0, 0.0, 0.0, 0.0};
  for (int k0 = 0; k0 < nt; k0 += 32) {
    for (int l = 0; l < 4; l++) {
      const int rr = ty + 8 * l, m = tm * 32 + tx, k = k0 + rr;
      // As[k][m] = op(A)(m, k)
      double va = 0.0;
      if (m < nt && k < nt) va = P.ta ? A[k + (long)m * nt] : A[m + (long)k * nt];
      As[rr][tx] = va;
      const int n = tn * 32 + rr, kb = k0 + tx;
      Bs[rr][tx] = (n < nt && kb < nt) ? Bm[kb + (long)n * nt] : 0.0;  // Bs[n][k]
    }
    __syncthreads();
    for (int k = 0; k < 32; k++)
      for (int l = 0; l < 4; l++) acc[l] = fma(As[k][tx], Bs[ty + 8 * l][k], acc[l]);
    __syncthreads();
  }
  for (int l = 0; l < 4; l++) {
    const int m = tm * 32 + tx, n = tn * 32 + ty + 8 * l;
    if (m < nt && n < nt) Y[P.y + m + (long)n * nt] = acc[l];
  }
}

// the transformed block back into the six arrays (:591-597)
__global__ void k_hf_scatter(const HfBlock2 *blks, const long *gam_off, const int *gam_n1, const int *gam_n2,
                             const double *Vn, double *H) {
  const HfBlock2 B = blks[blockIdx.x];
  const int nh = B.nh, nb = B.nb, nt = B.nt;
  // (g, row start, column start) of each array inside the square matrix
  const int r0[6] = {nh + nb, nh + nb, nh + nb, nh, 0, nh};
  const int c0[6] = {nh + nb, nh, 0, nh, 0, 0};
  for (int g = 0; g < 6; g++) {
    const long sg = (long)B.q * 6 + g;
    const int n1 = gam_n1[sg], n2 = gam_n2[sg];
    for (long e = threadIdx.x; e < (long)n1 * n2; e += blockDim.x) {
      const int i = (int)(e % n1), j = (int)(e / n1);
      H[gam_off[sg] + e] = Vn[B.off + (r0[g] + i) + (long)(c0[g] + j) * nt];
    }
  }
}

template <typename T>
int up(const std::vector<T> &h, T **d) {
  *d = nullptr;
  if (h.empty()) return IMSRG_OK;
  IMSRG_CUDA_TRY(cudaMalloc((void **)d, h.size() * sizeof(T)));
  IMSRG_CUDA_TRY(cudaMemcpy(*d, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice));
  return IMSRG_OK;
}

// device buffers of one Hartree-Fock call, freed on every return path
struct HfScratch {
  std::vector<void *> p;
  ~HfScratch() {
    for (void *x : p) cudaFree(x);
  }
  template <typename T>
  int upload(const std::vector<T> &h, T **d) {
    int s = up(h, d);
    if (*d) p.push_back(*d);
    return s;
  }
  template <typename T>
  int zeros(size_t n, T **d) {
    *d = nullptr;
    IMSRG_CUDA_TRY(cudaMalloc((void **)d, std::max<size_t>(n, 1) * sizeof(T)));
    p.push_back(*d);
    IMSRG_CUDA_TRY(cudaMemset(*d, 0, std::max<size_t>(n, 1) * sizeof(T)));
    return IMSRG_OK;
  }
};

// flat index of the one-body element <a|f|c> (f_elem) and whether it is
// stored transposed
long f_index(const imsrg_basis *b, const std::vector<int> &pos, int a, int c, bool *tr) {
  const int ca = b->con[a], cc = b->con[c];
  *tr = false;
  if (ca + cc == 0) return b->off_fpp + pos[a] + (long)pos[c] * b->P;
  if (ca + cc == 2) return b->off_fhh + pos[a] + (long)pos[c] * b->A;
  if (ca > cc) {
    *tr = true;
    return b->off_fph + pos[c] + (long)pos[a] * b->P;
  }
  return b->off_fph + pos[a] + (long)pos[c] * b->P;
}

std::vector<int> orbit_positions(const imsrg_basis *b) {
  std::vector<int> pos(b->norb);
  for (size_t k = 0; k < b->holes.size(); k++) pos[b->holes[k]] = (int)k;
  for (size_t k = 0; k < b->parts.size(); k++) pos[b->parts[k]] = (int)k;
  return pos;
}

// (l, j, tz) blocks in the reference's order (allocate_sp_mat,
// basic_IMSRG.f90:2600-2660): tz, l, j; their states in orbit order
int sp_blocks(const imsrg_basis *b, std::vector<SpBlock> &blk, std::vector<int> &states) {
  int lmax = 0, S = 0;
  for (int i = 0; i < b->norb; i++) lmax = std::max(lmax, b->ll[i]);
  blk.clear();
  states.clear();
  for (int tz = -1; tz <= 1; tz += 2)
    for (int l = 0; l <= lmax; l++)
      for (int j2 = 1; j2 <= b->jtm; j2 += 2) {
        SpBlock B{0, S, j2, (int)states.size()};
        for (int i = 0; i < b->norb; i++)
          if (b->ll[i] == l && b->jj[i] == j2 && b->itzp[i] == tz) {
            states.push_back(i);
            B.n++;
          }
        if (B.n > HF_MAXN) return IMSRG_ERR_TOO_LARGE;
        blk.push_back(B);
        S += B.n * B.n;
      }
  return IMSRG_OK;
}

// a block's matrix M (n x n, column-major at M + B.off) into the one-body
// part of the flat layout as transform_1b_to_HF (HF_mod.f90:460-487) places it
void place_onebody(const imsrg_basis *b, const std::vector<int> &pos, const std::vector<int> &states,
                   const SpBlock &B, const double *M, std::vector<double> &h) {
  for (int a = 0; a < B.n; a++)
    for (int c = a; c < B.n; c++) {
      const int i = states[B.st0 + a], j = states[B.st0 + c];
      bool tr;
      if (b->con[i] == b->con[j]) {
        h[f_index(b, pos, i, j, &tr)] = M[B.off + a + c * B.n];
        h[f_index(b, pos, j, i, &tr)] = M[B.off + a + c * B.n];
      } else if (b->con[j] > b->con[i]) {
        h[f_index(b, pos, i, j, &tr)] = M[B.off + a + c * B.n];
      } else {
        h[f_index(b, pos, j, i, &tr)] = M[B.off + c + a * B.n];
      }
    }
}

// transform_2b_to_HF (HF_mod.f90:494-619) of the two-body part of Hd in
// place with the coefficients Dsm (norb x norb, column-major): per block
// V' = E^T V E, E = C - (-1)^J Crev, two grouped GEMM launches
int transform_2b(imsrg_basis *b, double *Hd, const std::vector<double> &Dsm, cudaStream_t st) {
  std::vector<HfBlock2> b2;
  std::vector<int2> pairs;
  std::vector<HfGemm> g1, g2;
  long woff = 0;
  int tiles = 0;
  for (int q = 0; q < b->nblocks; q++) {
    const int nh = b->nhh[q], nb = b->nph[q], np = b->npp[q], nt = nh + nb + np;
    if (nt == 0) continue;
    HfBlock2 B{q, nh, nb, np, nt, woff, (int)pairs.size(), ((q / 6) & 1) ? -1 : 1};
    for (int c : {2, 1, 0}) {
      const std::vector<int> &qn = b->qn[q * 3 + c];
      for (size_t k = 0; k + 1 < qn.size(); k += 2) pairs.push_back(make_int2(qn[k], qn[k + 1]));
    }
    b2.push_back(B);
    const int t1 = (nt + 31) / 32;
    g1.push_back({woff, woff, woff, nt, 0, tiles, t1});  // Tmp = Vf E
    g2.push_back({woff, woff, woff, nt, 1, tiles, t1});  // Vn = E^T Tmp
    tiles += t1 * t1;
    woff += (long)nt * nt;
  }
  if (b2.empty()) return IMSRG_OK;
  HfScratch sc;
  HfBlock2 *d_b2;
  int2 *d_pairs;
  HfGemm *d_g1, *d_g2;
  double *d_Dsm, *d_V, *d_E, *d_Tmp;
  int *d_jj;
  std::vector<int> jjv(b->jj.begin(), b->jj.end());
  IMSRG_TRY(sc.upload(b2, &d_b2));
  IMSRG_TRY(sc.upload(pairs, &d_pairs));
  IMSRG_TRY(sc.upload(g1, &d_g1));
  IMSRG_TRY(sc.upload(g2, &d_g2));
  IMSRG_TRY(sc.upload(Dsm, &d_Dsm));
  IMSRG_TRY(sc.upload(jjv, &d_jj));
  IMSRG_TRY(sc.zeros(woff, &d_V));
  IMSRG_TRY(sc.zeros(woff, &d_E));
  IMSRG_TRY(sc.zeros(woff, &d_Tmp));
  std::vector<long> goff(b->gam_off.begin(), b->gam_off.end());
  std::vector<int> gn1(b->gam_n1.begin(), b->gam_n1.end()), gn2(b->gam_n2.begin(), b->gam_n2.end());
  long *d_goff;
  int *d_gn1, *d_gn2;
  IMSRG_TRY(sc.upload(goff, &d_goff));
  IMSRG_TRY(sc.upload(gn1, &d_gn1));
  IMSRG_TRY(sc.upload(gn2, &d_gn2));
  const int n2b = (int)b2.size();
  k_hf_vfull<<<n2b, 256, 0, st>>>(d_b2, d_goff, d_gn1, Hd, d_pairs, d_Dsm, b->norb, d_jj, d_V, d_E);
  k_hf_gemm<<<tiles, 256, 0, st>>>(d_g1, n2b, d_V, d_E, d_Tmp);
  k_hf_gemm<<<tiles, 256, 0, st>>>(d_g2, n2b, d_E, d_Tmp, d_V);
  k_hf_scatter<<<n2b, 256, 0, st>>>(d_b2, d_goff, d_gn1, d_gn2, d_V, Hd);
  b->launches += 4;
  IMSRG_CUDA_TRY(cudaGetLastError());
  return cuda_status(cudaStreamSynchronize(st));  // before the scratch is freed
}

}  // namespace
}  // namespace imsrg

using namespace imsrg;

extern "C" int imsrg_gpu_read_interaction(imsrg_op_t *H, const char *path, int htype, double hw, double com_hw,
                                          double lawson_beta, int mass) {
  IMSRG_TRY(op_ok(H));
  if (!path || H->herm != 1 || !(hw > 0.0) || mass <= 0) return IMSRG_ERR_INVALID;
  imsrg_basis *b = H->b;
  FILE *f = std::fopen(path, "r");
  if (!f) return IMSRG_ERR_IO;
  std::vector<double> h(b->nfull, 0.0);
  char line[4096];
  int nline = 0, status = IMSRG_OK;
  const int N = b->norb;
  const double cm2 = com_hw * com_hw / (hw * hw);
  while (std::fgets(line, sizeof line, f)) {
    if (++nline <= 8) continue;  // the header
    bool blank = true;
    for (const char *p = line; *p; p++)
      if (*p != ' ' && *p != '\t' && *p != '\n' && *p != '\r') blank = false;
    if (blank) continue;
    int Tz, Par, J2, a, bb, c, d;
    double V;
    if (std::sscanf(line, "%d %d %d %d %d %d %d %lf", &Tz, &Par, &J2, &a, &bb, &c, &d, &V) != 8) {
      status = IMSRG_ERR_IO;
      break;
    }
    a--, bb--, c--, d--;
    if (J2 < 0 || (J2 & 1)) {
      status = IMSRG_ERR_IO;
      break;
    }
    if (a < 0 || bb < 0 || c < 0 || d < 0 || a >= N || bb >= N || c >= N || d >= N) {
      status = IMSRG_ERR_INVALID;
      break;
    }
    // the element's block must be the one the line names
    const HLoc L = v_location(b, a, bb, c, d, J2);
    if (L.idx < 0 || Tz != (b->itzp[a] + b->itzp[bb]) / 2 || Par != (b->ll[a] + b->ll[bb]) % 2) {
      status = IMSRG_ERR_IO;
      break;
    }
    const double g2 = r1r2_p1p2(b, a, bb, c, d, J2, false), g3 = r1r2_p1p2(b, a, bb, c, d, J2, true);
    const double g1 = (g3 + cm2 * g2) * lawson_beta;
    V = V + (g1 - g3 * (htype == 1 ? 1.0 : 0.0)) * hw / mass;
    const double v = L.neg ? -V : V;
    h[L.idx] = v;
    // square arrays (pppp, phph, hhhh) hold both orders
    const int C1 = b->con[a] + b->con[bb], C2 = b->con[c] + b->con[d];
    if (C1 == C2) h[v_location(b, c, d, a, bb, J2).idx] = v;
  }
  std::fclose(f);
  if (status != IMSRG_OK) return status;
  IMSRG_CUDA_TRY(cudaMemcpyAsync(H->d, h.data(), b->nfull * sizeof(double), cudaMemcpyHostToDevice, b->stream));
  return cuda_status(cudaStreamSynchronize(b->stream));
}

extern "C" int imsrg_gpu_h0_harm_osc(imsrg_op_t *H, int htype, double hw, double com_hw, double lawson_beta,
                                     int mass) {
  IMSRG_TRY(op_ok(H));
  if (htype < 1 || htype > 5 || mass <= 0) return IMSRG_ERR_INVALID;
  imsrg_basis *b = H->b;
  const long o0 = b->off_fhh, o1 = b->off_2b;  // the one-body region
  std::vector<double> h(o1 - o0, 0.0);
  const std::vector<int> pos = orbit_positions(b);
  auto del = [](int x, int y) { return x == y ? 1.0 : 0.0; };
  for (int i = 0; i < b->norb; i++)
    for (int j = i; j < b->norb; j++) {
      if (b->ll[i] != b->ll[j] || b->jj[i] != b->jj[j] || b->itzp[i] != b->itzp[j]) continue;
      const int ni = b->nn[i], nj = b->nn[j], lj = b->ll[j];
      if (std::abs(ni - nj) > 1) continue;
      // HO kinetic matrix elements.  The reference writes the square roots
      // with default-REAL literals (nj*(nj+lj+0.5)), so they are single
      // precision; kept so, for the same numbers
      double kij;
      if (ni == nj) kij = 0.5 * hw * (2 * nj + lj + 1.5);
      else if (ni == nj - 1) kij = 0.5 * hw * (double)std::sqrt((float)nj * ((float)(nj + lj) + 0.5f));
      else kij = 0.5 * hw * (double)std::sqrt((float)(nj + 1) * ((float)(nj + lj) + 1.5f));
      const double hcm = kij * (del(ni, nj) - del(ni, nj + 1) - del(ni, nj - 1)) / mass;
      double T;
      switch (htype) {
        case 1:
          // the reference's order of operations
          T = std::fabs(lawson_beta) < 1e-5 ? kij * (1.0 - 1.0 / mass)
                                             : kij * (1.0 + (lawson_beta - 1.0) / mass) +
                                                   lawson_beta * com_hw * com_hw / (hw * hw) * kij *
                                                       (del(ni, nj) - del(ni, nj + 1) - del(ni, nj - 1)) / mass;
          break;
        case 2: T = 2 * kij * del(ni, nj); break;
        case 3: T = kij; break;
        case 4: T = kij / mass; break;
        default: T = hcm; break;
      }
      bool tr;
      h[f_index(b, pos, i, j, &tr) - o0] = T;
      if (b->con[i] == b->con[j]) h[f_index(b, pos, j, i, &tr) - o0] = T;
    }
  IMSRG_CUDA_TRY(cudaMemcpyAsync(H->d + o0, h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice, b->stream));
  return cuda_status(cudaStreamSynchronize(b->stream));
}

extern "C" int imsrg_gpu_hartree_fock(imsrg_op_t *H, double tol, int max_iter, double *e_hf, int *iterations,
                                      double *coefs) {
  IMSRG_TRY(op_ok(H));
  if (H->herm != 1 || max_iter <= 0 || !(tol > 0.0)) return IMSRG_ERR_INVALID;
  imsrg_basis *b = H->b;
  const int N = b->norb;
  cudaStream_t st = b->stream;
  IMSRG_CUDA_TRY(cudaStreamSynchronize(st));
  const std::vector<int> pos = orbit_positions(b);
  std::vector<SpBlock> blk;
  std::vector<int> states, eig_off;
  IMSRG_TRY(sp_blocks(b, blk, states));
  int S = 0, ne = 0;
  for (const SpBlock &B : blk) {
    eig_off.push_back(ne);
    S += B.n * B.n;
    ne += B.n;
  }
  const int nblk = (int)blk.size();
  // T from the operator's one-body part (write_kin_matrix, :138-166)
  std::vector<double> hop(b->nfull);
  IMSRG_CUDA_TRY(cudaMemcpy(hop.data(), H->d, b->nfull * sizeof(double), cudaMemcpyDeviceToHost));
  std::vector<double> Th(S, 0.0), Dh(S, 0.0);
  for (const SpBlock &B : blk)
    for (int i = 0; i < B.n; i++) {
      Dh[B.off + i + i * B.n] = 1.0;  // the HO reference
      for (int j = 0; j < B.n; j++) {
        bool tr;
        const int a = states[B.st0 + i], c = states[B.st0 + j];
        Th[B.off + i + j * B.n] = hop[f_index(b, pos, a, c, &tr)];  // herm +1: no sign
      }
    }
  // the Fock terms: element (q, i <= j) sums over every block qr and (g, h)
  std::vector<int> estart{0};
  std::vector<int2> epos;
  std::vector<HfTerm> terms;
  for (const SpBlock &B : blk)
    for (int i = 0; i < B.n; i++)
      for (int j = i; j < B.n; j++) {
        const int n1 = states[B.st0 + i], n3 = states[B.st0 + j];
        for (const SpBlock &R : blk)
          for (int g = 0; g < R.n; g++)
            for (int hh = 0; hh < R.n; hh++) {
              const int n2 = states[R.st0 + g], n4 = states[R.st0 + hh];
              for (int JJ = std::abs(R.j2 - B.j2); JJ <= R.j2 + B.j2; JJ += 2) {
                const HLoc L = v_location(b, n1, n2, n3, n4, JJ);
                if (L.idx < 0) continue;
                double c = (JJ + 1.0) / (R.j2 + 1.0) / (B.j2 + 1.0);
                if (L.neg) c = -c;
                for (int s = 0; s < L.nsq; s++) c *= 1.4142135623730951;
                terms.push_back({R.off + hh + g * R.n, L.idx, c});
              }
            }
        estart.push_back((int)terms.size());
        epos.push_back(make_int2(B.off + i + j * B.n, B.off + j + i * B.n));
      }
  const int nelem = (int)epos.size();
  std::vector<int> conv(b->con.begin(), b->con.end());
  HfScratch sc;
  SpBlock *d_blk;
  int *d_states, *d_con, *d_estart, *d_eigoff;
  int2 *d_epos;
  HfTerm *d_terms;
  double *d_T, *d_D, *d_rho, *d_G, *d_F, *d_eig;
  IMSRG_TRY(sc.upload(blk, &d_blk));
  IMSRG_TRY(sc.upload(states, &d_states));
  IMSRG_TRY(sc.upload(conv, &d_con));
  IMSRG_TRY(sc.upload(estart, &d_estart));
  IMSRG_TRY(sc.upload(epos, &d_epos));
  IMSRG_TRY(sc.upload(terms, &d_terms));
  IMSRG_TRY(sc.upload(eig_off, &d_eigoff));
  IMSRG_TRY(sc.upload(Th, &d_T));
  IMSRG_TRY(sc.upload(Dh, &d_D));
  IMSRG_TRY(sc.zeros(S, &d_rho));
  IMSRG_TRY(sc.zeros(S, &d_G));
  IMSRG_TRY(sc.zeros(S, &d_F));
  IMSRG_TRY(sc.zeros(ne, &d_eig));
  // the HF iterations (:51-72): density, potential, Fock matrix, eigenvectors
  std::vector<double> eig_old(ne, 0.0), eig_new(ne);
  int it = 0;
  double crit = 10.0;
  while (crit > tol) {
    if (it == max_iter) return IMSRG_ERR_NOT_CONVERGED;
    k_hf_density<<<nblk, 64, 0, st>>>(d_blk, nblk, d_states, d_con, d_D, d_rho);
    if (nelem) k_hf_gamma<<<(nelem + 3) / 4, 128, 0, st>>>(d_estart, d_epos, nelem, d_terms, d_rho, H->d, d_G);
    k_hf_diag<<<(nblk + 31) / 32, 32, 0, st>>>(d_blk, nblk, d_T, d_G, d_D, d_eig, d_eigoff);
    b->launches += 3;
    IMSRG_CUDA_TRY(cudaGetLastError());
    IMSRG_CUDA_TRY(cudaMemcpyAsync(eig_new.data(), d_eig, ne * sizeof(double), cudaMemcpyDeviceToHost, st));
    IMSRG_CUDA_TRY(cudaStreamSynchronize(st));
    crit = 0.0;  // fixed order, as the reference
    for (int q = 0; q < nblk; q++) {
      double s = 0.0;
      for (int i = 0; i < blk[q].n; i++) {
        const double x = eig_old[eig_off[q] + i] - eig_new[eig_off[q] + i];
        s += x * x;
      }
      crit += std::sqrt(s);
    }
    eig_old = eig_new;
    it++;
  }
  // sign convention and the one-body transformations (:74-91, :408-491)
  k_hf_transform1<<<(nblk + 31) / 32, 32, 0, st>>>(d_blk, nblk, d_D, d_T, d_G, d_F);
  b->launches++;
  IMSRG_CUDA_TRY(cudaGetLastError());
  std::vector<double> Fh(S), Tt(S), Gt(S);
  IMSRG_CUDA_TRY(cudaMemcpyAsync(Fh.data(), d_F, S * sizeof(double), cudaMemcpyDeviceToHost, st));
  IMSRG_CUDA_TRY(cudaMemcpyAsync(Tt.data(), d_T, S * sizeof(double), cudaMemcpyDeviceToHost, st));
  IMSRG_CUDA_TRY(cudaMemcpyAsync(Gt.data(), d_G, S * sizeof(double), cudaMemcpyDeviceToHost, st));
  IMSRG_CUDA_TRY(cudaMemcpyAsync(Dh.data(), d_D, S * sizeof(double), cudaMemcpyDeviceToHost, st));
  IMSRG_CUDA_TRY(cudaStreamSynchronize(st));
  // e_HF (:376-405) in the HF basis
  double ehf = 0.0;
  for (const SpBlock &B : blk)
    for (int i = 0; i < B.n; i++)
      ehf += (Tt[B.off + i + i * B.n] + 0.5 * Gt[B.off + i + i * B.n]) * b->con[states[B.st0 + i]] * (B.j2 + 1.0);
  // the Fock matrix in the HF basis is the new one-body part
  std::vector<double> Dsm((size_t)N * N, 0.0);
  for (long k = b->off_fhh; k < b->off_2b; k++) hop[k] = 0.0;
  for (const SpBlock &B : blk) {
    for (int a = 0; a < B.n; a++)
      for (int c = 0; c < B.n; c++) Dsm[states[B.st0 + a] + (size_t)states[B.st0 + c] * N] = Dh[B.off + a + c * B.n];
    place_onebody(b, pos, states, B, Fh.data(), hop);
  }
  hop[0] = ehf;
  IMSRG_CUDA_TRY(cudaMemcpyAsync(H->d, hop.data(), b->off_2b * sizeof(double), cudaMemcpyHostToDevice, st));
  // the two-body transformation, block by block (:494-619)
  IMSRG_TRY(transform_2b(b, H->d, Dsm, st));
  IMSRG_CUDA_TRY(cudaStreamSynchronize(st));
  if (e_hf) *e_hf = ehf;
  if (iterations) *iterations = it;
  if (coefs) std::memcpy(coefs, Dsm.data(), Dsm.size() * sizeof(double));
  return IMSRG_OK;
}

extern "C" int imsrg_gpu_transform_to_hf(imsrg_op_t *Op, const double *coefs) {
  IMSRG_TRY(op_ok(Op));
  if (!coefs || Op->herm != 1) return IMSRG_ERR_INVALID;
  imsrg_basis *b = Op->b;
  const int N = b->norb;
  cudaStream_t st = b->stream;
  const std::vector<int> pos = orbit_positions(b);
  std::vector<SpBlock> blk;
  std::vector<int> states;
  IMSRG_TRY(sp_blocks(b, blk, states));
  std::vector<double> Dsm(coefs, coefs + (size_t)N * N);
  // write_kin_matrix and transform_1b_to_HF (HF_mod.f90:108-136): the
  // one-body part block by block, X' = D^T X D, on the host (a few matrices
  // of at most HF_MAXN rows); zero across blocks
  std::vector<double> h(b->off_2b);
  IMSRG_CUDA_TRY(cudaMemcpyAsync(h.data(), Op->d, b->off_2b * sizeof(double), cudaMemcpyDeviceToHost, st));
  IMSRG_CUDA_TRY(cudaStreamSynchronize(st));
  std::vector<double> M;
  std::vector<double> out(h);
  for (long k = b->off_fhh; k < b->off_2b; k++) out[k] = 0.0;
  for (const SpBlock &B : blk) {
    const int n = B.n;
    if (n == 0) continue;
    std::vector<double> X(n * n), D(n * n), Y(n * n, 0.0);
    for (int i = 0; i < n; i++)
      for (int j = 0; j < n; j++) {
        bool tr;
        X[i + j * n] = h[f_index(b, pos, states[B.st0 + i], states[B.st0 + j], &tr)];
        D[i + j * n] = Dsm[states[B.st0 + i] + (size_t)states[B.st0 + j] * N];
      }
    M.assign(B.off + n * n, 0.0);
    for (int i = 0; i < n; i++)  // Y = X D
      for (int j = 0; j < n; j++)
        for (int k = 0; k < n; k++) Y[i + j * n] += X[i + k * n] * D[k + j * n];
    for (int i = 0; i < n; i++)  // D^T Y
      for (int j = 0; j < n; j++) {
        double s = 0.0;
        for (int k = 0; k < n; k++) s += D[k + i * n] * Y[k + j * n];
        M[B.off + i + j * n] = s;
      }
    place_onebody(b, pos, states, B, M.data(), out);
  }
  IMSRG_CUDA_TRY(cudaMemcpyAsync(Op->d, out.data(), b->off_2b * sizeof(double), cudaMemcpyHostToDevice, st));
  IMSRG_TRY(transform_2b(b, Op->d, Dsm, st));
  // normal ordering with respect to the HF reference
  return imsrg_gpu_normal_order(Op);
}
