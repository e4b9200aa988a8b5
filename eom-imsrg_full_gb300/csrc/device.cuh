// device.cuh -- device-side element access shared by the kernels.
//
// Device restatements of the reference accessors (n-parzuchowski/EOM-IMSRG_FULL,
// im-SRG/basic_IMSRG.f90): f_elem (:1147-1177), v_elem (:1270-1385),
// v_same (:2007-2028), sixj (:2509-2555).  v_same's COMMON-block cache becomes
// an explicit VLoc value: a location is resolved once and read from several
// operators.
#pragma once

#include "internal.h"

namespace imsrg {

__device__ __forceinline__ bool dtri(int j1, int j2, int J) { return J <= j1 + j2 && J >= abs(j1 - j2); }
__device__ __forceinline__ double m1pow(int e) { return (e & 1) ? -1.0 : 1.0; }

#define IMSRG_SQRT2 1.4142135623730951

// x * (-1)^neg by flipping the sign bit on the integer pipe (GB300's FP64
// pipe is the scarce resource; a DMUL by +-1 would occupy it).
__device__ __forceinline__ double dflip(double x, int neg) {
  return __longlong_as_double(__double_as_longlong(x) ^ ((unsigned long long)(neg & 1) << 63));
}

struct VLoc {
  long idx;  // flat index, -1 when the element is structurally zero
  int neg;   // phase (-1)^neg of the pair reorderings
  int nsq;   // number of sqrt(2) normalisation factors (a == b, c == d)
  int trans; // element read transposed: multiply by the operator's herm
};

__device__ __forceinline__ int pair_row(const DevTables &T, int a, int b, int J2) {
  return T.pairrow[((long)a * T.norb + b) * T.nJ + (J2 >> 1)];
}

// Location of <ab;J|V|cd;J> (orbits 0-based, J2 doubled).
__device__ __forceinline__ VLoc v_loc(const DevTables &T, int a, int b, int c, int d, int J2) {
  VLoc r;
  r.idx = -1;
  r.neg = 0;
  r.nsq = 0;
  r.trans = 0;
  int4 oa = T.orb[a], ob = T.orb[b], oc = T.orb[c], od = T.orb[d];
  if (!(dtri(oa.x, ob.x, J2) && dtri(oc.x, od.x, J2))) return r;
  int P = (oa.y + ob.y) & 1;
  if (((oc.y + od.y) & 1) != P) return r;
  int tz2 = oa.z + ob.z;
  if (oc.z + od.z != tz2) return r;
  int q = 3 * J2 + 2 * (tz2 / 2 + 1) + P;
  int C1 = oa.w + ob.w + 1, C2 = oc.w + od.w + 1;
  int qx = C1 * C2;
  if (qx == 9) qx = 5;
  int i1, i2;
  if (a > b) {
    i1 = pair_row(T, b, a, J2);
    r.neg = (1 + (oa.x + ob.x - J2) / 2) & 1;
  } else {
    r.nsq += (a == b);
    i1 = pair_row(T, a, b, J2);
  }
  if (c > d) {
    i2 = pair_row(T, d, c, J2);
    r.neg ^= (1 + (oc.x + od.x - J2) / 2) & 1;
  } else {
    r.nsq += (c == d);
    i2 = pair_row(T, c, d, J2);
  }
  int s = q * 6 + qx - 1;
  if (C1 > C2) {
    r.idx = T.gam_off[s] + i2 + (long)i1 * T.gam_n1[s];
    r.trans = 1;
  } else {
    r.idx = T.gam_off[s] + i1 + (long)i2 * T.gam_n1[s];
  }
  return r;
}

// Value at a location: op * (herm if transposed) * phase * sqrt(2)^nsq, with
// the sqrt(2) products rounded as the reference's pre * sqrt(2) chain.
__device__ __forceinline__ double v_read(const double *op, int herm, const VLoc &l) {
  if (l.idx < 0) return 0.0;
  double x = dflip(op[l.idx], l.neg ^ (l.trans & (herm < 0)));
  if (l.nsq) x = x * (l.nsq == 1 ? IMSRG_SQRT2 : 2.0000000000000004);
  return x;
}

__device__ __forceinline__ double v_elem(const DevTables &T, const double *op, int herm, int a, int b, int c, int d,
                                         int J2) {
  return v_read(op, herm, v_loc(T, a, b, c, d, J2));
}

__device__ __forceinline__ double f_elem(const DevTables &T, const double *op, int herm, int a, int b) {
  int ca = T.orb[a].w, cb = T.orb[b].w;
  int pa = T.orbpos[a], pb = T.orbpos[b];
  int s = ca + cb;
  if (s == 0) return op[T.off_fpp + pa + (long)pb * T.P];
  if (s == 2) return op[T.off_fhh + pa + (long)pb * T.A];
  if (ca > cb) return dflip(op[T.off_fph + pb + (long)pa * T.P], herm < 0);
  return op[T.off_fph + pa + (long)pb * T.P];
}

__device__ __forceinline__ long sixj_index(const DevTables &T, int j1, int j2, int J3, int j4, int j5, int J6) {
  return ((((long)(j1 >> 1) * T.nj + (j2 >> 1)) * T.nj + (j4 >> 1)) * T.nj + (j5 >> 1)) * T.nJ * T.nJ +
         (J3 >> 1) * T.nJ + (J6 >> 1);
}

// {j1 j2 J3; j4 j5 J6}: j1,j2,j4,j5 doubled half-integers, J3,J6 doubled integers.
__device__ __forceinline__ double sixj(const DevTables &T, int j1, int j2, int J3, int j4, int j5, int J6) {
  return T.six[sixj_index(T, j1, j2, J3, j4, j5, J6)];
}

// (J6 + 1) {j1 j2 J3; j4 j5 J6}, the weighted symbol of the Pandya transform.
__device__ __forceinline__ double sixj_w(const DevTables &T, int j1, int j2, int J3, int j4, int j5, int J6) {
  return T.six_w[sixj_index(T, j1, j2, J3, j4, j5, J6)];
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Sum of v over the CTA in a fixed order (warp shuffles, then the warp totals
// by the first warp), valid in the first warp; sh holds 32 doubles.
__device__ __forceinline__ double block_sum_ops(double v, double *sh) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0) sh[w] = v;
  __syncthreads();
  double r = 0.0;
  if (threadIdx.x < 32) {
    r = (lane < (int)(blockDim.x >> 5)) ? sh[lane] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) r += __shfl_xor_sync(0xffffffffu, r, o);
  }
  __syncthreads();
  return r;
}

}  // namespace imsrg
