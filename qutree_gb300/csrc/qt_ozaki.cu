// qt_ozaki.cu -- mode products of the double-float plans on the tensor cores.
//
// out[b, j, c] = alpha sum_a h(j, a) in[b, a, c] as Y = X H^T with rows
// r = (b, c): X is R x a_in, H^T is a_in x a_out (a_in, a_out <= 64).
// Each operand value v (double-float: hi + lo) is written against the
// exponent E of its row of X (resp. its row j of h) as an integer
//   m = trunc(v 2^(49 - E)),  |v| < 2^E,
// cut into seven 7-bit digits q_s (sign-magnitude, q_0 most significant):
//   v = 2^E sum_s q_s 2^(-7 (s + 1)) + (truncation below 2^(E - 49)).
// Every digit is an integer of magnitude <= 128, exact in bf16; a digit
// product is exact, and the sum over a_in <= 64 products of one level
// L = s + t of (at most seven) digit pairs stays below 2^23, so the tensor
// core's fp32 accumulation is exact.  The levels L = 0..6 (pairs with
// s + t > 6 fall below the 2^-49 truncation) are scaled by 2^(-7 (L + 2))
// and summed in double-float, then multiplied by 2^(E_r + F_j) and alpha.
// The error is below ~2^-48 of |row max of X| |row max of h| per product
// term, the order of double-float rounding.  Complex products use four real
// digit products (re re, im im, re im, im re).
//
// Warp-level mma.sync (m16n8k16, bf16 -> f32): a block of four warps takes
// 32 rows x 64 columns; each warp 16 rows x 32 columns (four n-fragments).
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "qt_arith.cuh"
#include "qt_internal.h"

namespace qt {
namespace {

constexpr int kOzRows = kMpOzRows;  // rows (b, c) per block
constexpr int kOzK = 64;            // largest a_in
constexpr int kOzN = kMpOzN;        // largest a_out
constexpr int kOzDig = kMpOzDig;    // digits per value
constexpr int kOzPitch = kMpOzPitch;  // bf16 elements per row (conflict-free fragment loads)
constexpr int kOzThreads = 128;

struct OzH {  // digits of h (global, one per task; copied to shared memory)
  uint16_t hd[kOzDig][2][kOzN][kOzPitch];  // [digit][re/im][j][k]
  int fx[kOzN];                            // row exponents of h (biased float exponent max)
};
struct OzSmem {
  OzH h;
  uint16_t xd[kOzDig][2][kOzRows][kOzPitch];  // digits of X: [digit][re/im][row][k]
  int ex[kOzRows];                            // row exponents of X
};
static_assert(sizeof(OzH) == 7 * 2 * 64 * 72 * 2 + 64 * 4, "OzH layout");

__device__ __forceinline__ int fexp(float v) { return (__float_as_int(v) >> 23) & 0xff; }

// 2^k as a float for -126 <= k <= 127
__device__ __forceinline__ float pow2f(int k) { return __int_as_float((k + 127) << 23); }

// v * 2^k exactly (the result is far from overflow and underflow), k in [-252, 254]
__device__ __forceinline__ float scale2(float v, int k) {
  if (k > 127) return (v * pow2f(127)) * pow2f(k - 127);
  if (k < -126) return (v * pow2f(-126)) * pow2f(k + 126);
  return v * pow2f(k);
}

// digits of hi + lo against exponent E (|hi + lo| < 2^E): 7 x 7 bits, with
// 32-bit integer and float operations only.  In units of 2^(E - 28) the
// value is I + fr (|fr| < 1): the four top digits come from the integer I,
// the three low ones from trunc(fr 2^21); the two parts carry their own
// signs, and v = 2^E sum_s q_s 2^(-7 (s + 1)) up to 2^(E - 49).
__device__ __forceinline__ void digits(float hi, float lo, int E, uint16_t* dst, int stride) {
  const float x1 = scale2(hi, 28 - E), y1 = scale2(lo, 28 - E);
  const float A = truncf(x1), B = truncf(y1);
  float fr = (x1 - A) + (y1 - B);
  const float tt = truncf(fr);
  const int I = (int)A + (int)B + (int)tt;
  fr -= tt;
  const int F = (int)truncf(scale2(fr, 21));
  const unsigned uI = (unsigned)(I < 0 ? -I : I), uF = (unsigned)(F < 0 ? -F : F);
  const float sI = I < 0 ? -1.f : 1.f, sF = F < 0 ? -1.f : 1.f;
  const unsigned q[kOzDig] = {uI >> 21, (uI >> 14) & 127u, (uI >> 7) & 127u, uI & 127u,
                              (uF >> 14) & 127u, (uF >> 7) & 127u, uF & 127u};
#pragma unroll
  for (int s = 0; s < kOzDig; ++s) {
    const float f = (s < 4 ? sI : sF) * (float)q[s];
    dst[s * stride] = __bfloat16_as_ushort(__float2bfloat16_rn(f));
  }
}

__device__ __forceinline__ void mma_bf16(float c[4], const uint32_t a[4], uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// pre-pass of a stage: the digits of h of every tensor-core task
__global__ void __launch_bounds__(256) k_mp_oz_h(const MPTask* __restrict__ tasks, const int* __restrict__ ids,
                                                 int64_t first) {
  const MPTask t = tasks[ids[first + blockIdx.x]];
  OzH* o = reinterpret_cast<OzH*>(t.oz_h);
  const float4* __restrict__ h = reinterpret_cast<const float4*>(t.h);
  const int K = t.a_in, N = t.a_out;
  const int Kp = (K + 15) & ~15;
  __shared__ int fx[kOzN];
  for (int i = threadIdx.x; i < kOzN; i += blockDim.x) fx[i] = 0;
  __syncthreads();
  for (int e = threadIdx.x; e < N * K; e += blockDim.x) {
    const int j = e % N, a = e / N;
    const float4 v = h[j + (int64_t)N * a];
    atomicMax(&fx[j], max(fexp(v.x), fexp(v.z)));
  }
  __syncthreads();
  for (int e = threadIdx.x; e < kOzN * kOzPitch; e += blockDim.x) {
    const int j = e / kOzPitch, a = e % kOzPitch;
    float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
    if (j < N && a < K) v = h[j + (int64_t)N * a];
    if (a < Kp || a >= kOzPitch) {
      const int F = fx[j] - 126;
      digits(v.x, v.y, F, &o->hd[0][0][j][a], 2 * kOzN * kOzPitch);
      digits(v.z, v.w, F, &o->hd[0][1][j][a], 2 * kOzN * kOzPitch);
    } else {
      for (int d = 0; d < kOzDig; ++d) o->hd[d][0][j][a] = o->hd[d][1][j][a] = 0;
    }
  }
  for (int i = threadIdx.x; i < kOzN; i += blockDim.x) o->fx[i] = fx[i];
}

__global__ void __launch_bounds__(kOzThreads) k_mp_oz(const MPTask* __restrict__ tasks,
                                                      const int2* __restrict__ tiles, int64_t tile0) {
  extern __shared__ __align__(16) unsigned char oz_raw[];
  OzSmem& sm = *reinterpret_cast<OzSmem*>(oz_raw);
  const int2 tl = tiles[tile0 + blockIdx.x];
  const MPTask t = tasks[tl.x];
  const float4* __restrict__ in = reinterpret_cast<const float4*>(t.in);
  const float4* __restrict__ h = reinterpret_cast<const float4*>(t.h);
  float4* out = reinterpret_cast<float4*>(t.out);
  const int K = t.a_in, N = t.a_out;
  const int64_t before = t.before;
  const int64_t nrows = before * t.after;
  const int64_t row0 = (int64_t)tl.y * kOzRows;
  const int tid = threadIdx.x;
  const int Kp = (K + 15) & ~15;

  // digits of h: written by the stage's pre-pass, copied with 16-byte loads
  {
    const uint4* src = reinterpret_cast<const uint4*>(t.oz_h);
    uint4* dst = reinterpret_cast<uint4*>(&sm.h);
    for (int i = tid; i < (int)(sizeof(OzH) / 16); i += kOzThreads) dst[i] = src[i];
  }
  for (int i = tid; i < kOzRows; i += kOzThreads) sm.ex[i] = 0;
  __syncthreads();
  const bool rows_fast = before > 1;  // consecutive rows are adjacent in memory
  for (int e = tid; e < kOzRows * K; e += kOzThreads) {
    const int rl = rows_fast ? e % kOzRows : e / K, a = rows_fast ? e / kOzRows : e % K;
    const int64_t r = row0 + rl;
    if (r >= nrows) continue;
    const int64_t b = r % before, c = r / before;
    const float4 v = in[b + before * a + before * K * c];
    atomicMax(&sm.ex[rl], max(fexp(v.x), fexp(v.z)));
  }
  __syncthreads();
  for (int e = tid; e < kOzRows * Kp; e += kOzThreads) {
    const int rl = rows_fast ? e % kOzRows : e / Kp, a = rows_fast ? e / kOzRows : e % Kp;
    const int64_t r = row0 + rl;
    float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
    if (r < nrows && a < K) {
      const int64_t b = r % before, c = r / before;
      v = in[b + before * a + before * K * c];
    }
    const int E = sm.ex[rl] - 126;
    digits(v.x, v.y, E, &sm.xd[0][0][rl][a], 2 * kOzRows * kOzPitch);
    digits(v.z, v.w, E, &sm.xd[0][1][rl][a], 2 * kOzRows * kOzPitch);
  }
  __syncthreads();

  const int warp = tid >> 5, lane = tid & 31;
  const int g = lane >> 2, q4 = lane & 3;
  const int rbase = 16 * (warp & 1), cbase = 32 * (warp >> 1);
  if (cbase >= N) return;
  // double-float sums per output: [n-fragment][element][re/im] (hi, lo)
  float shi[4][4][2], slo[4][4][2];
#pragma unroll
  for (int f = 0; f < 4; ++f)
#pragma unroll
    for (int e = 0; e < 4; ++e)
#pragma unroll
      for (int z = 0; z < 2; ++z) shi[f][e][z] = slo[f][e][z] = 0.f;

  for (int L = 0; L < kOzDig; ++L) {
    float rr[4][4], ii[4][4], ri[4][4], ir[4][4];
#pragma unroll
    for (int f = 0; f < 4; ++f)
#pragma unroll
      for (int e = 0; e < 4; ++e) rr[f][e] = ii[f][e] = ri[f][e] = ir[f][e] = 0.f;
    for (int s = 0; s <= L; ++s) {
      const int u = L - s;
      for (int kk = 0; kk < Kp; kk += 16) {
        uint32_t xr[4], xi[4];
        const uint16_t* pr = &sm.xd[s][0][rbase + g][kk + 2 * q4];
        const uint16_t* pi = &sm.xd[s][1][rbase + g][kk + 2 * q4];
        xr[0] = *reinterpret_cast<const uint32_t*>(pr);
        xr[1] = *reinterpret_cast<const uint32_t*>(pr + 8 * kOzPitch);
        xr[2] = *reinterpret_cast<const uint32_t*>(pr + 8);
        xr[3] = *reinterpret_cast<const uint32_t*>(pr + 8 * kOzPitch + 8);
        xi[0] = *reinterpret_cast<const uint32_t*>(pi);
        xi[1] = *reinterpret_cast<const uint32_t*>(pi + 8 * kOzPitch);
        xi[2] = *reinterpret_cast<const uint32_t*>(pi + 8);
        xi[3] = *reinterpret_cast<const uint32_t*>(pi + 8 * kOzPitch + 8);
#pragma unroll
        for (int f = 0; f < 4; ++f) {
          const uint16_t* qr = &sm.h.hd[u][0][cbase + 8 * f + g][kk + 2 * q4];
          const uint16_t* qi = &sm.h.hd[u][1][cbase + 8 * f + g][kk + 2 * q4];
          const uint32_t hr0 = *reinterpret_cast<const uint32_t*>(qr);
          const uint32_t hr1 = *reinterpret_cast<const uint32_t*>(qr + 8);
          const uint32_t hi0 = *reinterpret_cast<const uint32_t*>(qi);
          const uint32_t hi1 = *reinterpret_cast<const uint32_t*>(qi + 8);
          mma_bf16(rr[f], xr, hr0, hr1);
          mma_bf16(ii[f], xi, hi0, hi1);
          mma_bf16(ri[f], xr, hi0, hi1);
          mma_bf16(ir[f], xi, hr0, hr1);
        }
      }
    }
    // level L: exact integer sums -> scaled into the double-float sums
    const float sc = pow2f(-7 * (L + 2));
#pragma unroll
    for (int f = 0; f < 4; ++f)
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        const float yr = (rr[f][e] - ii[f][e]) * sc;
        const float yi = (ri[f][e] + ir[f][e]) * sc;
        df_add(shi[f][e][0], slo[f][e][0], yr, 0.f);
        df_add(shi[f][e][1], slo[f][e][1], yi, 0.f);
      }
  }
  // scale by 2^(E_r + F_j), times alpha, store
  const float4 alpha = DF64::coef(t.alpha);
  const bool unit = t.alpha.x == 1.0 && t.alpha.y == 0.0;
#pragma unroll
  for (int f = 0; f < 4; ++f)
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const int rl = rbase + g + 8 * (e >> 1);
      const int j = cbase + 8 * f + 2 * q4 + (e & 1);
      const int64_t r = row0 + rl;
      if (r >= nrows || j >= N) continue;
      const int sh = (sm.ex[rl] - 126) + (sm.h.fx[j] - 126);
      float4 v;
      v.x = scale2(shi[f][e][0], sh);
      v.y = scale2(slo[f][e][0], sh);
      v.z = scale2(shi[f][e][1], sh);
      v.w = scale2(slo[f][e][1], sh);
      df_norm(v.x, v.y);
      df_norm(v.z, v.w);
      if (!unit) v = DF64::mul(alpha, v);
      const int64_t b = r % before, c = r / before;
      out[b + before * j + before * (int64_t)N * c] = v;
    }
}

}  // namespace

cudaError_t launch_mp_oz(const MPTask* tasks, const int2* tiles, int64_t first_tile, int64_t n_tiles,
                         const int* oz_tasks, int64_t first_task, int64_t n_tasks, cudaStream_t s) {
  if (n_tiles <= 0) return cudaSuccess;
  if (n_tasks > 0) k_mp_oz_h<<<(unsigned)n_tasks, 256, 0, s>>>(tasks, oz_tasks, first_task);
  const int sm = (int)sizeof(OzSmem);
  cudaError_t e = cudaFuncSetAttribute(k_mp_oz, cudaFuncAttributeMaxDynamicSharedMemorySize, sm);
  if (e != cudaSuccess) return e;
  k_mp_oz<<<(unsigned)n_tiles, kOzThreads, sm, s>>>(tasks, tiles, first_tile);
  return cudaGetLastError();
}

}  // namespace qt
