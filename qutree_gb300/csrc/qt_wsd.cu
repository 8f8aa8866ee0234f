// qt_wsd.cu -- weighted simultaneous diagonalisation of the CDVR grids
// (LayerGrid with several matrices, src/DVR/TDDVR.cpp:72-88, around
// WeightedSimultaneousDiagonalization::calculate,
// src/Util/WeightedSimultaneousDiagonalization.cpp:5-378, and the Jacobi
// rotation helpers of src/Core/JacobiRotationFramework.cpp:4-164).
//
// One block of four warps per problem.  The iteration accepts or rejects
// optimiser steps on comparisons of nearly equal numbers, so its result is a
// discontinuous function of the inputs; this file therefore fixes one
// operation order, which the CPU restatement follows bit for bit:
//  * compiled with -fmad=false: no multiply-add is fused; a complex product
//    is (ac - bd) + i(ad + bc) (a Givens rotation's real c multiplies both
//    parts alone), sums run left to right; a sum over the
//    matrices of a problem is the pairwise tree of the values padded with
//    zeros to a power of two, and the measure adds its per-matrix traces in
//    index order;
//  * |z| is sqrt(re^2 + im^2); real(x / w) is (xr wr + xi wi) / (wr^2 + wi^2);
//    the rotated diagonals of a candidate rotation use the Hermitian form
//    c^2 A_pp + 2c Re(s A_pq) + |s|^2 A_qq (c is real);
//  * the optimiser's 3x3 eigenvector (Matrix::rDiag) comes from the largest
//    root of the characteristic polynomial of H scaled by a power of two
//    (binary32 Newton from the Gershgorin bound, then binary64 Newton from
//    that root plus 2^-17 with binary32 step quotients, until a step is
//    below 2^-30) and the largest cross product of two rows of H - lambda.
//
// Execution on this GPU: an FP64 operation has ~32 ns of latency and a
// division or square root ~0.3 us, whatever the number of active lanes, and
// the optimiser is one long dependency chain of them (thousands of
// candidate evaluations per problem, in sequence).  So:
//  * warp 0 (the master) runs the optimiser's scalar chain; every lane holds
//    the same values, and independent divisions / square roots of the chain
//    go to different lanes of ONE instruction (results fetched by shuffles)
//    instead of one after another;
//  * all four warps run the parallel phases (rotated diagonals of every
//    matrix at ten candidate rotations, the level-by-level tree sums,
//    Givens rotations of every matrix, the products of the off-diagonality
//    measure).  The loops are the same in every warp; the master publishes
//    each loop decision in shared memory before the barrier that precedes
//    it, so the barriers match by construction;
//  * the matrices live in shared memory when they fit (else in the task's
//    global scratch).
// All loops are bounded (at most 25 sweeps, 30 optimiser iterations, 64 step
// halvings per search, 40 + 100 Newton steps).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "qt_internal.h"

namespace qt {
namespace {

constexpr int kWsdThreads = 128;
constexpr unsigned kFull = 0xffffffffu;
constexpr int kWsdSmemBudget = 220 * 1024;

__device__ __forceinline__ double2 cm(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ double2 ca(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 cs(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ double2 cc(double2 a) { return make_double2(a.x, -a.y); }
// product with the real c of a rotation: (c x.re, c x.im)
__device__ __forceinline__ double2 rm(double2 c, double2 a) { return make_double2(c.x * a.x, c.x * a.y); }
__device__ __forceinline__ double cabs_(double2 a) { return sqrt(a.x * a.x + a.y * a.y); }
__device__ __forceinline__ double cdiv_re(double2 x, double2 w) {
  return (x.x * w.x + x.y * w.y) / (w.x * w.x + w.y * w.y);
}
__device__ __forceinline__ void bsync() { __syncthreads(); }

// binary64 -> binary32 by truncation of the significand; zero below 2^-126,
// infinity above the binary32 range (integer operations only)
__device__ __forceinline__ float f32_trunc(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const unsigned sign = (unsigned)(b >> 32) & 0x80000000u;
  const int e = (int)((b >> 52) & 0x7ff) - 896;
  unsigned r;
  if (e <= 0)
    r = sign;
  else if (e >= 255)
    r = sign | 0x7f800000u;
  else
    r = sign | ((unsigned)e << 23) | (unsigned)((b >> 29) & 0x7fffffu);
  return __uint_as_float(r);
}
// binary32 -> binary64, exact for normal numbers; subnormals become zero
__device__ __forceinline__ double f64_of(float f) {
  const unsigned r = __float_as_uint(f);
  const unsigned long long sign = (unsigned long long)(r & 0x80000000u) << 32;
  const unsigned e = (r >> 23) & 0xffu;
  unsigned long long b;
  if (e == 0)
    b = sign;
  else if (e == 255)
    b = sign | 0x7ff0000000000000ull | ((unsigned long long)(r & 0x7fffffu) << 29);
  else
    b = sign | ((unsigned long long)(e + 896) << 52) | ((unsigned long long)(r & 0x7fffffu) << 29);
  return __longlong_as_double((long long)b);
}

struct Prob {
  int d, n;
  int H, lgH;  // first level of the matrix tree: H = max(P2 / 2, 1) = 2^lgH, P2 = n padded to a power of two
  int chunk;   // matrices per pass of the off-diagonality measure
  double2* xw;  // n weighted matrices
  double2* xp;  // n plain (shifted) matrices
  double2* w;   // weight
  double2* T;   // transformation
  double2* tM;  // chunk x d^2: X T, then Y Y
  double2* tY;  // chunk x d^2: Y
  double2* blk;   // (n + 1) x 4: (pp, pq, qp, qq) of every matrix and of w at the current pair
  double2* cand;  // 10 x 2: candidate (c, s)
  double2* rot;   // the accepted rotation (c, s) of the pair
  double* sq;     // two tree buffers of 2 x 10 x H
  double* wd;     // 10 x 2: rotated diagonals of w per candidate
  double* tr;     // chunk x d: diagonal of W Z per matrix
  double* val;    // 2: broadcast values
  int* ctl;       // 2: loop decisions
  const uint32_t* lut;  // kEigLevels x 32 lane descriptors
  __device__ double2* X(int k) const { return xw + (int64_t)k * d * d; }
  __device__ double2* Xp(int k) const { return xp + (int64_t)k * d * d; }
};

// ---- master warp: the optimiser's scalar chain --------------------------------

// ---- lane-vectorised evaluation ------------------------------------------------
// An FP64 instruction occupies the SM sub-partition's FP64 unit for the same
// time whether or not it depends on the previous one, so the scalar chain
// costs one unit slot per instruction.  Independent multiplies, adds and
// subtracts of one level therefore go into ONE fused multiply-add across
// the lanes: x*y as fma(x, y, -0), x + y as fma(1, x, y), x - y as
// fma(1, x, -y) -- each rounds exactly once, like the separate operation
// (the -0 addend keeps the sign of a zero product).  A level's operands are
// shuffled from a slot vector S (lane l holds value #l); lane descriptors
// (shared memory, one 32-bit word per lane and level) name the source slots,
// the operation, |y| and whether the lane keeps its result.

// -x and |x| on the sign bit (integer instructions, the IEEE results)
__device__ __forceinline__ double neg_bits(double x) {
  return __longlong_as_double(__double_as_longlong(x) ^ (long long)0x8000000000000000ull);
}
__device__ __forceinline__ double abs_bits(double x) {
  return __longlong_as_double(__double_as_longlong(x) & 0x7fffffffffffffffll);
}

enum { OP_MUL = 0, OP_ADD = 1, OP_SUB = 2 };
constexpr uint32_t lane_desc(int x, int y, int op, int absy = 0) {
  return (uint32_t)x | ((uint32_t)y << 5) | ((uint32_t)op << 10) | ((uint32_t)absy << 12) | (1u << 13);
}
__device__ __forceinline__ double fma_op(int op, double x, double y) {
  const double f = op == OP_MUL ? x : 1.0;
  const double g = op == OP_MUL ? y : x;
  const double h = op == OP_MUL ? -0.0 : (op == OP_ADD ? y : neg_bits(y));
  return __fma_rn(f, g, h);
}
__device__ __forceinline__ double lane_level(double S, uint32_t dsc) {
  const double x = __shfl_sync(kFull, S, dsc & 31);
  double y = __shfl_sync(kFull, S, (dsc >> 5) & 31);
  if (dsc & (1u << 12)) y = abs_bits(y);
  const double r = fma_op((dsc >> 10) & 3, x, y);
  return (dsc >> 13) & 1 ? r : S;
}
// Comparisons of binary64 values by their bits (integer instructions; the
// same truth values as the floating-point comparison, NaN included):
// x < 0; x > 0; x > c and x < c for a constant c > 0
__device__ __forceinline__ unsigned long long bits_of(double x) { return (unsigned long long)__double_as_longlong(x); }
__device__ __forceinline__ bool is_negative(double x) {
  const unsigned long long b = bits_of(x), mag = b & 0x7fffffffffffffffull;
  return (b >> 63) && mag != 0 && mag <= 0x7ff0000000000000ull;
}
__device__ __forceinline__ bool is_positive(double x) {
  const unsigned long long b = bits_of(x);
  return !(b >> 63) && b != 0 && b <= 0x7ff0000000000000ull;
}
__device__ __forceinline__ bool gt_pos(double x, double c) {
  const unsigned long long b = bits_of(x);
  return !(b >> 63) && b > bits_of(c) && b <= 0x7ff0000000000000ull;
}
__device__ __forceinline__ bool lt_pos(double x, double c) {
  const unsigned long long b = bits_of(x);
  return (b >> 63) ? ((b & 0x7fffffffffffffffull) <= 0x7ff0000000000000ull) : b < bits_of(c);
}
// a / 2 and a * 2 for a power of two a in the normal range: the exponent
__device__ __forceinline__ double half_pow2(double a) { return __longlong_as_double((long long)(bits_of(a) - (1ull << 52))); }
__device__ __forceinline__ double twice_pow2(double a) { return __longlong_as_double((long long)(bits_of(a) + (1ull << 52))); }

// p / dp as a call, so that the rare fallback of the Newton step is a branch
// and not an always-executed division
__device__ __noinline__ double exact_quotient(double p, double dp) { return p / dp; }

// Levels of the 3x3 eigenproblem.  Slots at entry: 0 h00, 1 h01, 2 h11,
// 3 h02, 4 h12, 5 h22 (= 0).
constexpr int kEigLevels = 11;
enum { EL_C1 = 0, EL_C2, EL_C3, EL_C4, EL_C5, EL_E1, EL_E2, EL_E3, EL_E4, EL_E5, EL_E6 };
__constant__ uint32_t c_eig_lut[kEigLevels][32] = {
    // C1: the products of m and det, (h00 + h11), the Gershgorin rows' first sums
    {0, 0, 0, 0, 0, 0, 0, 0,
     lane_desc(0, 2, OP_MUL), lane_desc(1, 1, OP_MUL), lane_desc(0, 5, OP_MUL), lane_desc(3, 3, OP_MUL),
     lane_desc(2, 5, OP_MUL), lane_desc(4, 4, OP_MUL), lane_desc(1, 5, OP_MUL), lane_desc(4, 3, OP_MUL),
     lane_desc(1, 4, OP_MUL), lane_desc(2, 3, OP_MUL), lane_desc(0, 2, OP_ADD), lane_desc(0, 1, OP_ADD, 1),
     lane_desc(2, 1, OP_ADD, 1), lane_desc(5, 3, OP_ADD, 1)},
    // C2: the three terms of m, the inner terms of det, tr, the Gershgorin rows
    {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0,
     lane_desc(8, 9, OP_SUB), lane_desc(10, 11, OP_SUB), lane_desc(12, 13, OP_SUB), lane_desc(14, 15, OP_SUB),
     lane_desc(16, 17, OP_SUB), lane_desc(18, 5, OP_ADD), lane_desc(19, 3, OP_ADD, 1), lane_desc(20, 4, OP_ADD, 1),
     lane_desc(21, 4, OP_ADD, 1)},
    // C3: the outer products of det, the first sum of m, 2 tr
    {0, 0, 0, 0, 0, 0, 0, 0, lane_desc(0, 24, OP_MUL), lane_desc(1, 25, OP_MUL), lane_desc(3, 26, OP_MUL),
     lane_desc(22, 23, OP_ADD), lane_desc(27, 27, OP_ADD)},
    // C4
    {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, lane_desc(8, 9, OP_SUB), lane_desc(11, 24, OP_ADD)},
    // C5: det
    {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, lane_desc(13, 10, OP_ADD)},
    // E1: m00, m11, m22 (lambda in slot 31)
    {0, 0, 0, 0, 0, 0, lane_desc(0, 31, OP_SUB), lane_desc(2, 31, OP_SUB), lane_desc(5, 31, OP_SUB)},
    // E2: the products of the three cross products (slots 6 m00, 7 m11, 8 m22)
    {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0,
     lane_desc(1, 4, OP_MUL), lane_desc(3, 7, OP_MUL), lane_desc(3, 1, OP_MUL), lane_desc(6, 4, OP_MUL),
     lane_desc(6, 7, OP_MUL), lane_desc(1, 1, OP_MUL), lane_desc(1, 8, OP_MUL), lane_desc(3, 4, OP_MUL),
     lane_desc(3, 3, OP_MUL), lane_desc(6, 8, OP_MUL), lane_desc(7, 8, OP_MUL), lane_desc(4, 4, OP_MUL)},
    // E3: components c01 (9..11), c02 (12..14), c12 (15..17)
    {0, 0, 0, 0, 0, 0, 0, 0, 0,
     lane_desc(16, 17, OP_SUB), lane_desc(18, 19, OP_SUB), lane_desc(20, 21, OP_SUB), lane_desc(22, 23, OP_SUB),
     lane_desc(24, 25, OP_SUB), lane_desc(19, 18, OP_SUB), lane_desc(26, 27, OP_SUB), lane_desc(23, 22, OP_SUB),
     lane_desc(16, 17, OP_SUB)},
    // E4: their squares (18..26)
    {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0,
     lane_desc(9, 9, OP_MUL), lane_desc(10, 10, OP_MUL), lane_desc(11, 11, OP_MUL), lane_desc(12, 12, OP_MUL),
     lane_desc(13, 13, OP_MUL), lane_desc(14, 14, OP_MUL), lane_desc(15, 15, OP_MUL), lane_desc(16, 16, OP_MUL),
     lane_desc(17, 17, OP_MUL)},
    // E5: v0^2 + v1^2 of each (27..29)
    {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0,
     lane_desc(18, 19, OP_ADD), lane_desc(21, 22, OP_ADD), lane_desc(24, 25, OP_ADD)},
    // E6: the squared norms (0..2)
    {lane_desc(27, 20, OP_ADD), lane_desc(28, 23, OP_ADD), lane_desc(29, 26, OP_ADD)},
};

// Matrix::rDiag of the optimiser's symmetric 3x3 matrix (rfoBuildHessian,
// src/Core/JacobiRotationFramework.cpp:114-127: h00 = pre0 a^2, h01 = pre2 a^2,
// h11 = pre3 a^2, h02 = grad0 a, h12 = grad1 a, h22 = 0): the eigenvector of
// the largest eigenvalue as u0 = v0/v2, u1 = v1/v2 and v0^2 + v1^2 for |v| = 1.
// Whole warp 0, every lane the same inputs and outputs.
__device__ void eig3_top(const uint32_t* lut, double p0, double p2, double p3, double g0, double g1, double a,
                         double* u0, double* u1, double* top2) {
  const int l = threadIdx.x & 31;
  double S = (l == 0 ? p0 : (l == 1 ? p2 : (l == 2 ? p3 : (l == 3 ? g0 : g1)))) * a;
  S = S * (l < 3 ? a : 1.0);
  {  // scale by 2^(1023 - e), e the largest biased exponent: max |entry| in [1, 2)
    int e = l < 5 ? (int)(((unsigned long long)__double_as_longlong(S) >> 52) & 0x7ff) : 0;
    e = __reduce_max_sync(kFull, e);
    if (e >= 1 && e <= 2045) S = S * __longlong_as_double((long long)(2046 - e) << 52);
  }
  if (l >= 5) S = 0.0;
  const double h00 = __shfl_sync(kFull, S, 0), h01 = __shfl_sync(kFull, S, 1), h11 = __shfl_sync(kFull, S, 2);
  const double h02 = __shfl_sync(kFull, S, 3), h12 = __shfl_sync(kFull, S, 4), h22 = 0.0;
  // tr = (h00 + h11) + h22; m and det as three terms each; Gershgorin rows
#pragma unroll
  for (int k = EL_C1; k <= EL_C5; ++k) S = lane_level(S, lut[k * 32 + l]);
  const double tr = __shfl_sync(kFull, S, 27), tr2 = __shfl_sync(kFull, S, 12);
  const double m = __shfl_sync(kFull, S, 14), det = __shfl_sync(kFull, S, 15);
  double lam_g = __shfl_sync(kFull, S, 28);
  const double r1 = __shfl_sync(kFull, S, 29), r2 = __shfl_sync(kFull, S, 30);
  if (r1 > lam_g) lam_g = r1;
  if (r2 > lam_g) lam_g = r2;
  // binary32 Newton from the Gershgorin bound: p(l) = -l^3 + tr l^2 - m l + det
  float fl = f32_trunc(lam_g);
  {
    const float f00 = f32_trunc(h00), f01 = f32_trunc(h01), f02 = f32_trunc(h02);
    const float f11 = f32_trunc(h11), f12 = f32_trunc(h12), f22 = f32_trunc(h22);
    const float ftr = f00 + f11 + f22;
    const float fm = (f00 * f11 - f01 * f01) + (f00 * f22 - f02 * f02) + (f11 * f22 - f12 * f12);
    const float fdet = f00 * (f11 * f22 - f12 * f12) - f01 * (f01 * f22 - f12 * f02) + f02 * (f01 * f12 - f11 * f02);
    for (int it = 0; it < 40; ++it) {
      const float p = ((-fl + ftr) * fl - fm) * fl + fdet;
      const float dp = (-3.0f * fl + 2.0f * ftr) * fl - fm;
      if (!(dp < 0.0f)) break;
      const float nx = fl - p / dp;
      if (!(nx < fl)) break;
      fl = nx;
    }
  }
  // binary64 Newton, monotone from above.  p = ((-lam + tr) lam - m) lam + det
  // in lane 0 and p' = (-3 lam + 2 tr) lam - m in lane 1, one instruction
  // per step of both chains; 3 lam in lane 2.
  double lam = f64_of(fl) + 0x1p-17;
  double p, dp, l3;
  const double neg_m = neg_bits(m);
  auto pdp = [&]() {
    double v = __fma_rn(l == 0 ? 1.0 : (l == 1 ? -3.0 : 3.0), l == 0 ? neg_bits(lam) : lam, l == 0 ? tr : -0.0);
    l3 = __shfl_sync(kFull, v, 2);
    v = __fma_rn(l == 1 ? 1.0 : v, l == 1 ? v : lam, l == 1 ? tr2 : -0.0);
    v = __fma_rn(l == 0 ? 1.0 : v, l == 0 ? v : lam, l == 0 ? neg_m : -0.0);
    v = __fma_rn(l == 0 ? v : 1.0, l == 0 ? lam : v, l == 0 ? -0.0 : neg_m);
    dp = __shfl_sync(kFull, v, 1);
    v = __fma_rn(1.0, v, det);
    p = __shfl_sync(kFull, v, 0);
  };
  pdp();
  if (!(is_negative(p) && is_negative(dp) && l3 > tr)) {
    lam = lam_g;
    pdp();
  }
  for (int it = 0; it < 100; ++it) {
    if (!is_negative(dp)) break;
    double step = f64_of(f32_trunc(p) / f32_trunc(dp));
    if (!(((unsigned long long)__double_as_longlong(step) & 0x7fffffffffffffffull) <= 0x4030000000000000ull))
      step = exact_quotient(p, dp);  // |step| > 16 or NaN: the binary32 quotient left its range
    const double nxt = lam - step;
    if (!(nxt < lam)) break;
    lam = nxt;
    // step > 0 here: compare the bits with those of 2^-30
    if ((unsigned long long)__double_as_longlong(step) <= 0x3e10000000000000ull) break;
    pdp();
  }
  // eigenvector: the largest cross product of two rows of H - lambda
  if (l == 31) S = lam;
#pragma unroll
  for (int k = EL_E1; k <= EL_E6; ++k) S = lane_level(S, lut[k * 32 + l]);
  const double n01 = __shfl_sync(kFull, S, 0), n02 = __shfl_sync(kFull, S, 1), n12 = __shfl_sync(kFull, S, 2);
  int sel = 0;
  double nv = n01;
  if (n02 > nv) {
    sel = 1;
    nv = n02;
  }
  if (n12 > nv) sel = 2;
  // u0 = v0 / v2, u1 = v1 / v2, top2 = (v0^2 + v1^2) / |v|^2 in lanes 0, 1, 2
  const double num = __shfl_sync(kFull, S, l == 0 ? 9 + 3 * sel : (l == 1 ? 10 + 3 * sel : 27 + sel));
  const double den = __shfl_sync(kFull, S, l < 2 ? 11 + 3 * sel : sel);
  const double r = num / den;
  *u0 = __shfl_sync(kFull, r, 0);
  *u1 = __shfl_sync(kFull, r, 1);
  *top2 = __shfl_sync(kFull, r, 2);
}

// weightedJacobiDerivatives from the loss at the nine points (i, j) of the
// central differences (y[i + 3 j]): lane k takes numerator k as
// ((A + B) - C) - D (a difference x - y as x + (-y); subtracting +0 keeps
// every value) and one division gives all five quotients
__device__ void grad_pre(const double y[9], double delta, double& g0, double& g1, double& p0, double& p2,
                         double& p3) {
  const int l = threadIdx.x & 31;
  const double y4x2 = 2 * y[1 + 3 * 1];
  const double A = l == 0 || l == 2 ? y[2 + 3 * 1] : (l == 1 || l == 3 ? y[1 + 3 * 2] : y[2 + 3 * 2]);
  const double B = l == 0 ? neg_bits(y[0 + 3 * 1])
                           : (l == 1 ? neg_bits(y[1 + 3 * 0]) : (l == 2 ? y[0 + 3 * 1] : (l == 3 ? y[1 + 3 * 0] : y[0 + 3 * 0])));
  const double C = l < 2 ? 0.0 : (l < 4 ? y4x2 : y[2 + 3 * 0]);
  const double D = l < 4 ? 0.0 : y[0 + 3 * 2];
  const double num = ((A + B) - C) - D;
  const double den = l < 2 ? 2 * delta : (l < 4 ? delta * delta : 4 * delta * delta);
  const double r = num / den;
  g0 = __shfl_sync(kFull, r, 0);
  g1 = __shfl_sync(kFull, r, 1);
  p0 = __shfl_sync(kFull, r, 2);
  p3 = __shfl_sync(kFull, r, 3);
  p2 = __shfl_sync(kFull, r, 4);
}

// Candidate 0 = (sqrt|arg0|, s) and the nine samples of the central
// differences around s (weightedJacobiDerivatives) into P.cand, one square
// root per lane (lanes 0..9); lane 10 takes sqrt|arg10|.  Returns each
// lane's root.
__device__ double put_candidates(const Prob& P, double arg0, double sx, double sy, double delta, double arg10) {
  const int l = threadIdx.x & 31;
  double x0 = sx, x1 = sy, arg = l == 10 ? arg10 : arg0;
  if (l >= 1 && l <= 9) {
    const int q = l - 1, i = q % 3, j = q / 3;
    // (i - 1) delta and (j - 1) delta: -delta, +0 or delta, exactly
    x0 = sx + (i == 0 ? -delta : (i == 1 ? 0.0 : delta));
    x1 = sy + (j == 0 ? -delta : (j == 1 ? 0.0 : delta));
    const double z = x0 * x0 + x1 * x1;
    arg = 1 - z;
  }
  const double r = sqrt(abs_bits(arg));
  if (l <= 9) {
    P.cand[2 * l] = make_double2(r, 0.0);
    P.cand[2 * l + 1] = make_double2(x0, x1);
  }
  return r;
}

// ---- parallel phases (all warps) ------------------------------------------------

// rotatedDiagonals of a cached 2x2 block (pp, pq, qp, qq) of a Hermitian
// matrix for a real c: a0 = c^2 A_pp + 2c Re(s A_pq) + |s|^2 A_qq and
// a1 = c^2 A_qq - 2c Re(s A_pq) + |s|^2 A_pp
__device__ __forceinline__ void rotated_diagonals(const double2* b, double2 c, double2 s, double& a0, double& a1) {
  const double cc2 = c.x * c.x;
  const double ss2 = s.x * s.x + s.y * s.y;
  const double c2 = 2.0 * c.x;
  const double2 apq = b[1];
  const double t = s.x * apq.x - s.y * apq.y;
  const double ct = c2 * t;
  a0 = (cc2 * b[0].x + ct) + ss2 * b[3].x;
  a1 = (cc2 * b[3].x - ct) + ss2 * b[0].x;
}

// levels 2.. of the pairwise tree over `count` rows of H values per
// component (level 1 is in buf); returns the buffer holding the sums
__device__ double* tree_levels(const Prob& P, int count) {
  const int H = P.H, tid = threadIdx.x;
  double* buf = P.sq;
  double* alt = P.sq + 2 * 10 * H;
  for (int lg = P.lgH; lg > 0; --lg) {  // sizes H, H/2, .., 2 (powers of two)
    const int half = 1 << (lg - 1);
    for (int it = tid; it < (2 * count) << (lg - 1); it += kWsdThreads) {
      const int g = it >> (lg - 1), i = it & (half - 1);  // g = (component, candidate)
      const int comp = g >= count ? 1 : 0, j = g - comp * count;
      const double* src = buf + comp * 10 * H + j * H;
      alt[comp * 10 * H + j * H + i] = src[2 * i] + src[2 * i + 1];
    }
    bsync();
    double* t = buf;
    buf = alt;
    alt = t;
  }
  return buf;
}

// weightedJacobiLoc for the `count` candidates in P.cand; xo0, xo1 = xold / w
// of the pair.  Returns, in warp 0, the loss change of candidate j in lane j
// and xnum / xden (a division of the caller's, issued with the same
// instruction) in lane 2 count.  Other warps return 0.
__device__ double loc_many(const Prob& P, int count, double xo0, double xo1, double xnum, double xden) {
  const int n = P.n, H = P.H, tid = threadIdx.x;
  const int items = count * H;
  // squared rotated diagonals with the first tree level; w's rotated diagonals
  for (int it = tid; it < items + count; it += kWsdThreads) {
    if (it < items) {
      const int j = it >> P.lgH, i = it & (H - 1);
      const double2 c = P.cand[2 * j], s = P.cand[2 * j + 1];
      double r0, r1, s0 = 0.0, s1 = 0.0;
      if (n == 1) {
        rotated_diagonals(P.blk, c, s, r0, r1);
        s0 = r0 * r0;
        s1 = r1 * r1;
      } else {
        double a0 = 0.0, a1 = 0.0, b0 = 0.0, b1 = 0.0;
        if (2 * i < n) {
          rotated_diagonals(P.blk + 8 * i, c, s, r0, r1);
          a0 = r0 * r0;
          a1 = r1 * r1;
        }
        if (2 * i + 1 < n) {
          rotated_diagonals(P.blk + 8 * i + 4, c, s, r0, r1);
          b0 = r0 * r0;
          b1 = r1 * r1;
        }
        s0 = a0 + b0;
        s1 = a1 + b1;
      }
      P.sq[j * H + i] = s0;
      P.sq[10 * H + j * H + i] = s1;
    } else {
      const int j = it - items;
      double r0, r1;
      rotated_diagonals(P.blk + 4 * n, P.cand[2 * j], P.cand[2 * j + 1], r0, r1);
      P.wd[2 * j] = r0;
      P.wd[2 * j + 1] = r1;
    }
  }
  bsync();
  const double* sums = tree_levels(P, count);
  double res = 0.0;
  if (tid < 32) {  // diff = (xnew0 / w0 - xold0 / w_pp) + (xnew1 / w1 - xold1 / w_qq), one division per lane
    const int l = tid;
    double num = xnum, den = xden;
    if (l < 2 * count) {
      const int c = l >= count ? 1 : 0, j = l - c * count;
      num = sums[c * 10 * H + j * H];
      den = P.wd[2 * j + c];
    }
    const double q = num / den;
    const double t = q - (l < count ? xo0 : xo1);
    const double t1 = __shfl_sync(kFull, t, (l + count) & 31);
    double diff = 0;
    diff += t;
    diff += t1;
    res = l < count ? diff : q;
  }
  return res;
}

// calculateWeightedAngles: rational function optimisation of (c, s).  The
// loss of every new candidate is evaluated together with the nine samples of
// the central differences around it: if the candidate is accepted they are
// the next iteration's derivatives, if not the derivatives at the unchanged
// point are still valid -- the same numbers the reference recomputes.
// All threads; the rotation is returned in warp 0.
__device__ void angles(const Prob& P, double xo0, double xo1, double2& c_out, double2& s_out) {
  const bool master = threadIdx.x < 32;
  const int lane = threadIdx.x & 31;
  const double eps = 1E-3, amin = 1E-12, amax = 1, delta = 1E-5;
  double a = amax, diff_rel = 2 * eps * eps;
  double c0 = 0, s0 = eps, s1 = -eps, sab = 0, loc_alt = 0;
  double ycur[9];
  if (master) {
    const double r = put_candidates(P, 1 - 2 * eps * eps, s0, s1, delta, s0 * s0 + s1 * s1);
    c0 = __shfl_sync(kFull, r, 0);
    sab = __shfl_sync(kFull, r, 10);  // |s|
  }
  bsync();
  {
    const double res = loc_many(P, 10, xo0, xo1, 0.0, 1.0);
    if (master) {
      loc_alt = __shfl_sync(kFull, res, 0);
#pragma unroll
      for (int q = 0; q < 9; ++q) ycur[q] = __shfl_sync(kFull, res, 1 + q);
    }
  }
  for (int iter = 0; iter < 30; ++iter) {
    if (master && lane == 0) P.ctl[0] = (gt_pos(diff_rel, eps * eps) && gt_pos(a, amin)) ? 1 : 0;
    bsync();
    if (!P.ctl[0]) break;
    double g0 = 0, g1 = 0, p0 = 0, p2 = 0, p3 = 0;
    if (master) grad_pre(ycur, delta, g0, g1, p0, p2, p3);
    double diff = -1, loc_new = 0, cnew = 0, snew0 = 0, snew1 = 0, zab = 0, top2 = 0;
    double ynew[9];
#pragma unroll
    for (int q = 0; q < 9; ++q) ynew[q] = 0;
    for (int guard = 0; guard < 64; ++guard) {
      if (master) {
        const int go = (gt_pos(a, amin) && is_negative(diff) && gt_pos(diff_rel, eps * eps)) ? 1 : 0;
        if (go) {
          double z = 1;
          for (int g2 = 0; gt_pos(a, amin) && gt_pos(z, 0.5) && g2 < 64; ++g2) {
            // rfoBuildHessian (src/Core/JacobiRotationFramework.cpp:114-127)
            double u0, u1;
            eig3_top(P.lut, p0, p2, p3, g0, g1, a, &u0, &u1, &top2);
            // ds = a u, snew = s + ds in lanes 0 and 1; zab = sqrt(snew0^2 + snew1^2)
            double v = a * (lane == 0 ? u0 : u1);
            v = (lane == 0 ? s0 : s1) + v;
            snew0 = __shfl_sync(kFull, v, 0);
            snew1 = __shfl_sync(kFull, v, 1);
            v = v * v;
            zab = sqrt(__shfl_sync(kFull, v, 0) + __shfl_sync(kFull, v, 1));
            z = zab * zab;
            if (gt_pos(z, 0.5)) a = half_pow2(a);
          }
          const double r = put_candidates(P, 1 - z, snew0, snew1, delta, 0.0);
          cnew = __shfl_sync(kFull, r, 0);
        }
        if (lane == 0) P.ctl[1] = go;
      }
      bsync();
      if (!P.ctl[1]) break;
      const double res = loc_many(P, 10, xo0, xo1, top2, sab * sab + eps * eps);
      if (master) {
        loc_new = __shfl_sync(kFull, res, 0);
#pragma unroll
        for (int q = 0; q < 9; ++q) ynew[q] = __shfl_sync(kFull, res, 1 + q);
        diff_rel = __shfl_sync(kFull, res, 20);  // |trafo|^2 / (|s|^2 + eps^2)
        diff = loc_new - loc_alt;
        if (is_negative(diff)) {
          a = half_pow2(a);
        } else {
          if (lt_pos(a, amax)) a = twice_pow2(a);
        }
      }
    }
    if (master && gt_pos(a, amin) && is_positive(diff)) {
      c0 = cnew;
      s0 = snew0;
      s1 = snew1;
      sab = zab;
      loc_alt = loc_new;
#pragma unroll
      for (int q = 0; q < 9; ++q) ycur[q] = ynew[q];
    }
  }
  c_out = make_double2(c0, 0.0);
  s_out = make_double2(s0, s1);
}

// weightedJacobiRotations: every pair (i < j) in order; for each, the
// optimised rotation applied to every weighted matrix, to w and to T
__device__ void rotations(const Prob& P) {
  const int d = P.d, n = P.n, H = P.H, tid = threadIdx.x;
  const bool master = tid < 32;
  for (int i = 0; i < d - 1; ++i)
    for (int j = i + 1; j < d; ++j) {
      // the (i, j) blocks of every matrix and of w; the squared current
      // diagonals with the first level of their tree
      for (int it = tid; it < n + 1 + H; it += kWsdThreads) {
        if (it <= n) {
          const double2* A = it < n ? P.X(it) : P.w;
          P.blk[4 * it + 0] = A[i + (int64_t)d * i];
          P.blk[4 * it + 1] = A[i + (int64_t)d * j];
          P.blk[4 * it + 2] = A[j + (int64_t)d * i];
          P.blk[4 * it + 3] = A[j + (int64_t)d * j];
        } else {
          const int h = it - n - 1;
          double s0, s1;
          if (n == 1) {
            const double x0 = P.X(0)[i + (int64_t)d * i].x, x1 = P.X(0)[j + (int64_t)d * j].x;
            s0 = x0 * x0;
            s1 = x1 * x1;
          } else {
            double a0 = 0.0, a1 = 0.0, b0 = 0.0, b1 = 0.0;
            if (2 * h < n) {
              const double x0 = P.X(2 * h)[i + (int64_t)d * i].x, x1 = P.X(2 * h)[j + (int64_t)d * j].x;
              a0 = x0 * x0;
              a1 = x1 * x1;
            }
            if (2 * h + 1 < n) {
              const double x0 = P.X(2 * h + 1)[i + (int64_t)d * i].x, x1 = P.X(2 * h + 1)[j + (int64_t)d * j].x;
              b0 = x0 * x0;
              b1 = x1 * x1;
            }
            s0 = a0 + b0;
            s1 = a1 + b1;
          }
          P.sq[h] = s0;
          P.sq[10 * H + h] = s1;
        }
      }
      bsync();
      const double* sums = tree_levels(P, 1);
      double xo0 = 0, xo1 = 0;
      if (master) {  // xold / w of the pair, lanes 0 and 1
        const int l = tid;
        const double r = (l == 0 ? sums[0] : sums[10 * H]) / (l == 0 ? P.blk[4 * n + 0].x : P.blk[4 * n + 3].x);
        xo0 = __shfl_sync(kFull, r, 0);
        xo1 = __shfl_sync(kFull, r, 1);
      }
      double2 c, s;
      angles(P, xo0, xo1, c, s);
      if (tid == 0) {
        P.rot[0] = c;
        P.rot[1] = s;
      }
      bsync();
      c = P.rot[0];
      s = P.rot[1];
      // givensRotation of every matrix and of w, columns i, j; givensTrafoRotation of T
      for (int e = tid; e < (n + 2) * d; e += kWsdThreads) {
        const int mi = e / d, r = e % d;
        if (mi <= n) {
          double2* B = mi < n ? P.X(mi) : P.w;
          const double2 bri = B[r + (int64_t)d * i], brj = B[r + (int64_t)d * j];
          B[r + (int64_t)d * i] = ca(rm(c, bri), cm(s, brj));
          B[r + (int64_t)d * j] = cs(rm(c, brj), cm(cc(s), bri));
        } else {
          const double2 ti = P.T[r + (int64_t)d * i], tj = P.T[r + (int64_t)d * j];
          P.T[r + (int64_t)d * i] = ca(rm(c, ti), cm(s, tj));
          P.T[r + (int64_t)d * j] = cs(rm(c, tj), cm(cc(s), ti));
        }
      }
      bsync();
      // rows i, j
      for (int e = tid; e < (n + 1) * d; e += kWsdThreads) {
        const int mi = e / d, r = e % d;
        double2* B = mi < n ? P.X(mi) : P.w;
        const double2 c0 = B[i + (int64_t)d * r], c1 = B[j + (int64_t)d * r];
        B[i + (int64_t)d * r] = ca(rm(c, c0), cm(cc(s), c1));
        B[j + (int64_t)d * r] = cs(rm(c, c1), cm(s, c0));
      }
      bsync();
    }
}

// measureWeightedOffDiagonality: sum_k Re tr(W (D_k - T^H X_k T)^2), the
// matrices `chunk` at a time, the elements of each product in parallel, each
// an ordered sum; the traces added in index order.  All threads get the sum.
__device__ double offdiag(const Prob& P) {
  const int d = P.d, n = P.n, tid = threadIdx.x;
  const int64_t dd = (int64_t)d * d;
  double total = 0;
  for (int k0 = 0; k0 < n; k0 += P.chunk) {
    const int cnt = P.chunk < n - k0 ? P.chunk : n - k0;
    for (int64_t e = tid; e < cnt * dd; e += kWsdThreads) {  // M = X T
      const int kk = (int)(e / dd);
      const int64_t ee = e % dd;
      const int i = (int)(ee % d), j = (int)(ee / d);
      const double2* X = P.Xp(k0 + kk);
      double2 acc = make_double2(0, 0);
      for (int l = 0; l < d; ++l) acc = ca(acc, cm(X[i + (int64_t)d * l], P.T[l + (int64_t)d * j]));
      P.tM[kk * dd + ee] = acc;
    }
    bsync();
    for (int64_t e = tid; e < cnt * dd; e += kWsdThreads) {  // Y = D - T^H M
      const int kk = (int)(e / dd);
      const int64_t ee = e % dd;
      const int i = (int)(ee % d), j = (int)(ee / d);
      const double2* M = P.tM + kk * dd;
      double2 acc = make_double2(0, 0);
      for (int l = 0; l < d; ++l) acc = ca(acc, cm(cc(P.T[l + (int64_t)d * i]), M[l + (int64_t)d * j]));
      double2 dg = make_double2(0, 0);
      if (i == j) dg = make_double2(cdiv_re(P.X(k0 + kk)[i + (int64_t)d * i], P.w[i + (int64_t)d * i]), 0);
      P.tY[kk * dd + ee] = cs(dg, acc);
    }
    bsync();
    for (int64_t e = tid; e < cnt * dd; e += kWsdThreads) {  // Z = Y Y
      const int kk = (int)(e / dd);
      const int64_t ee = e % dd;
      const int i = (int)(ee % d), j = (int)(ee / d);
      const double2* Y = P.tY + kk * dd;
      double2 acc = make_double2(0, 0);
      for (int l = 0; l < d; ++l) acc = ca(acc, cm(Y[i + (int64_t)d * l], Y[l + (int64_t)d * j]));
      P.tM[kk * dd + ee] = acc;
    }
    bsync();
    for (int e = tid; e < cnt * d; e += kWsdThreads) {  // Re (W Z)_ii
      const int kk = e / d, i = e % d;
      const double2* Z = P.tM + kk * dd;
      double2 acc = make_double2(0, 0);
      for (int l = 0; l < d; ++l) acc = ca(acc, cm(P.w[i + (int64_t)d * l], Z[l + (int64_t)d * i]));
      P.tr[e] = acc.x;
    }
    bsync();
    if (tid < 32) {  // trace of matrix k0 + b + lane, then the traces in index order
      for (int b = 0; b < cnt; b += 32) {
        double t = 0;
        if (b + tid < cnt)
          for (int i = 0; i < d; ++i) t += P.tr[(b + tid) * d + i];
        const int m = cnt - b < 32 ? cnt - b : 32;
        for (int q = 0; q < m; ++q) total += __shfl_sync(kFull, t, q);
      }
    }
  }
  if (tid == 0) P.val[0] = total;
  bsync();
  const double v = P.val[0];
  bsync();
  return v;
}

// shared memory of the fixed part of a problem with n matrices of order d
__host__ __device__ int64_t wsd_fixed_bytes(int n, int d) {
  int64_t p2 = 1;
  while (p2 < n) p2 <<= 1;
  const int64_t H = p2 > 1 ? p2 / 2 : 1;
  const int64_t b = 16 * (4 * (int64_t)(n + 1) + 20 + 2) + 8 * (40 * H + 20 + (int64_t)n * d + 2) + 16 +
                    4 * kEigLevels * 32;
  return (b + 15) / 16 * 16;
}

__global__ void __launch_bounds__(kWsdThreads, 1) k_wsd(const WSDTask* __restrict__ tasks,
                                                     const WSDTerm* __restrict__ terms, int64_t first,
                                                     int smem_bytes) {
  const WSDTask t = tasks[first + blockIdx.x];
  const int d = t.d, n = t.n;
  const int tid = threadIdx.x;
  const int64_t dd = (int64_t)d * d;
  extern __shared__ __align__(16) unsigned char wsd_smem[];
  Prob P;
  P.d = d;
  P.n = n;
  {
    int p2 = 1;
    while (p2 < n) p2 <<= 1;
    P.H = p2 > 1 ? p2 / 2 : 1;
    P.lgH = 0;
    while ((1 << P.lgH) < P.H) ++P.lgH;
  }
  P.blk = reinterpret_cast<double2*>(wsd_smem);
  P.cand = P.blk + 4 * (n + 1);
  P.rot = P.cand + 20;
  P.sq = reinterpret_cast<double*>(P.rot + 2);
  P.wd = P.sq + 40 * P.H;
  P.tr = P.wd + 20;
  P.val = P.tr + (int64_t)n * d;
  P.ctl = reinterpret_cast<int*>(P.val + 2);
  {
    uint32_t* lut = reinterpret_cast<uint32_t*>(P.ctl + 4);
    for (int i = tid; i < kEigLevels * 32; i += kWsdThreads) lut[i] = (&c_eig_lut[0][0])[i];
    P.lut = lut;
  }
  // the matrices in shared memory when they fit, else in the task's scratch
  const int64_t fixed = wsd_fixed_bytes(n, d);
  const int64_t mats = (2 * (int64_t)n + 2) * dd * 16;
  const int64_t room = (int64_t)smem_bytes - fixed - mats;
  if (room >= 2 * dd * 16) {
    double2* base = reinterpret_cast<double2*>(wsd_smem + fixed);
    const int64_t fit = room / (2 * dd * 16);
    P.chunk = fit < n ? (int)fit : n;
    P.xw = base;
    P.xp = base + n * dd;
    P.w = base + 2 * n * dd;
    P.T = P.w + dd;
    P.tM = P.T + dd;
    P.tY = P.tM + P.chunk * dd;
  } else {
    P.chunk = 1;
    P.xw = t.scratch;
    P.xp = t.scratch + n * dd;
    P.w = t.scratch + 2 * n * dd;
    P.T = P.w + dd;
    P.tM = P.T + dd;
    P.tY = P.tM + dd;
  }
  // w = regularize(W), T = 1
  for (int64_t e = tid; e < dd; e += kWsdThreads) {
    double2 v = t.W[e];
    const int i = (int)(e % d), j = (int)(e / d);
    if (i == j) v.x += 1e-9 * exp(-cabs_(v) / 1e-9);
    P.w[e] = v;
    P.T[e] = make_double2(i == j ? 1.0 : 0.0, 0.0);
  }
  // shifts |tr X| (calculateShift), kept in the grid's imaginary parts until the end
  for (int k = tid; k < n; k += kWsdThreads) {
    const double2* X = terms[t.first + k].X;
    double2 tr = make_double2(0, 0);
    for (int i = 0; i < d; ++i) tr = ca(tr, X[i + (int64_t)d * i]);
    const double sh = cabs_(tr);
    t.grid[(int64_t)k * d].y = sh;
    P.tr[k] = sh;
  }
  bsync();
  // plain matrices shifted (shift)
  for (int64_t e = tid; e < n * dd; e += kWsdThreads) {
    const int k = (int)(e / dd);
    const int64_t ee = e % dd;
    double2 v = terms[t.first + k].X[ee];
    if (ee % (d + 1) == 0) v.x -= P.tr[k];
    P.Xp(k)[ee] = v;
  }
  bsync();
  // weightMatrices: (X w + w X) / 2
  for (int64_t e = tid; e < (int64_t)n * dd; e += kWsdThreads) {
    const int k = (int)(e / dd);
    const int i = (int)(e % dd % d), j = (int)(e % dd / d);
    const double2* x = P.Xp(k);
    double2 xw = make_double2(0, 0), wx = make_double2(0, 0);
    for (int l = 0; l < d; ++l) {
      xw = ca(xw, cm(x[i + (int64_t)d * l], P.w[l + (int64_t)d * j]));
      wx = ca(wx, cm(P.w[i + (int64_t)d * l], x[l + (int64_t)d * j]));
    }
    const double2 sum = ca(xw, wx);
    P.X(k)[i + (int64_t)d * j] = make_double2(0.5 * sum.x, 0.5 * sum.y);
  }
  bsync();
  double delta = offdiag(P);
  int iter = 0;
  bool converged = false;
  const double eps = 1e-5;
  while (!converged && iter < 25) {
    rotations(P);
    const double delta_last = delta;
    delta = offdiag(P);
    const double change = fabs(delta_last - delta);
    if (delta < eps || change < eps) converged = true;
    iter++;
  }
  // grid = Re(Xw(i,i) / w(i,i)) + shift; trafo = T^dagger
  for (int k = tid; k < n; k += kWsdThreads) {
    const double sh = t.grid[(int64_t)k * d].y;
    for (int i = 0; i < d; ++i)
      t.grid[(int64_t)k * d + i] = make_double2(cdiv_re(P.X(k)[i + (int64_t)d * i], P.w[i + (int64_t)d * i]) + sh, 0.0);
  }
  for (int64_t e = tid; e < dd; e += kWsdThreads) {
    const int i = (int)(e % d), j = (int)(e / d);
    t.trafo[e] = cc(P.T[j + (int64_t)d * i]);
  }
}

}  // namespace

cudaError_t launch_wsd(const WSDTask* tasks, const WSDTerm* terms, int64_t first, int64_t n, int max_n,
                       int max_d, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  const int64_t dd = (int64_t)max_d * max_d;
  const int64_t fixed = wsd_fixed_bytes(max_n, max_d);
  if (fixed > kWsdSmemBudget) return cudaErrorInvalidValue;
  // the largest problem's matrices and as many per-matrix product buffers as fit
  const int64_t mats = (2 * (int64_t)max_n + 2) * dd * 16;
  int64_t sm = fixed;
  if (fixed + mats + 2 * dd * 16 <= kWsdSmemBudget)
    sm = std::min<int64_t>(fixed + mats + 2 * (int64_t)max_n * dd * 16,
                           fixed + mats + (kWsdSmemBudget - fixed - mats) / (2 * dd * 16) * (2 * dd * 16));
  cudaError_t e = cudaFuncSetAttribute(k_wsd, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  if (e != cudaSuccess) return e;
  k_wsd<<<(unsigned)n, kWsdThreads, sm, s>>>(tasks, terms, first, (int)sm);
  return cudaGetLastError();
}

}  // namespace qt
