// qt_ozaki.cu -- mode products of the double-float plans on the tensor cores.
//
// out[b, j, c] = alpha sum_a h(j, a) in[b, a, c] as Y = X H^T with rows
// r = (b, c): X is R x a_in, H^T is a_in x a_out (a_in, a_out <= 64).
// Each operand value v (double-float: hi + lo) is written against the
// exponent E of its row of X (resp. its row j of h) as an integer
//   m = round(v 2^(49 - E)),  |v| < 2^E,  |m| <= 2^49,
// cut into seven 7-bit digits q_s (sign-magnitude, q_0 most significant, at
// most 128): v = 2^E sum_s q_s 2^(-7 (s + 1)) within one unit of 2^(E - 49).
// Every digit is exact in bf16 and a digit product is exact.  Each level
// L = s + t <= 6 (pairs with s + t > 6 are dropped) keeps its own fp32 sums
// of re and im; the real part takes X_re H_re and
// (-X_im) H_im in one accumulator, at most 2 * 7 * 64 * 128^2 < 2^24 in
// magnitude, so the tensor core's fp32 sums are exact.  The levels are scaled
// by 2^(-7 (L + 2)), summed in double-float and multiplied by 2^(E_r + F_j)
// and alpha.  The error is below 2^-44 of |row max of X| |row max of h| per
// real product term (the dropped pairs s + t >= 7 and the rounding of both
// operands); measured errors sit near 2^-48 of it.
//
// Warp-level mma.sync (m16n8k16, bf16 -> f32) on fragments loaded with
// ldmatrix.  A pre-pass writes each task's digits of h once per stage.  A
// block of sixteen warps copies them into shared memory (cp.async, all in
// flight) and takes kMpOzSub sub-tiles of 32 rows x 64 columns, each warp a
// 16 x 8 tile.  The seven levels' sums stay in registers; the loops run digit
// s of X, k-step, digit u of h, so one A fragment serves every u, and the
// levels are combined once per sub-tile.  While the warps run the products of
// one sub-tile, the next sub-tile's X is already on its way into registers.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>

#include "qt_arith.cuh"
#include "qt_internal.h"

namespace qt {
namespace {

constexpr int kOzRows = kMpOzRows;  // rows (b, c) per sub-tile
constexpr int kOzSub = kMpOzSub;    // sub-tiles per block
constexpr int kOzK = 64;            // largest a_in
constexpr int kOzN = kMpOzN;        // largest a_out
constexpr int kOzDig = kMpOzDig;    // digits per value
constexpr int kOzPitch = kMpOzPitch;  // bf16 elements per row (conflict-free fragment loads)
constexpr int kOzThreads = 512;
constexpr int kOzPre = kOzRows * kOzK / kOzThreads;  // X values per thread per sub-tile

struct OzH {  // digits of h (global, one per task; copied to shared memory)
  uint16_t hd[kOzDig][2][kOzN][kOzPitch];  // [digit][re/im][j][k]
  int fx[kOzN];                            // row exponents of h (biased float exponent max)
};
struct OzSmem {
  OzH h;
  uint16_t xd[kOzDig][2][kOzRows][kOzPitch];  // digits of X: [digit][re/im][row][k]
  int ex[2][kOzRows];                         // row exponents of X (two sub-tiles), at least 1
  int64_t orow[2][kOzRows];                   // output offset of each row (-1: past the end)
};
static_assert(sizeof(OzH) == 7 * 2 * 64 * 72 * 2 + 64 * 4, "OzH layout");
static_assert(sizeof(OzH) % 16 == 0 && (kOzPitch * 2) % 16 == 0, "16-byte rows for cp.async and ldmatrix");

__device__ __forceinline__ int fexp(float v) { return (__float_as_int(v) >> 23) & 0xff; }

// 2^k as a float for -126 <= k <= 127
__device__ __forceinline__ float pow2f(int k) { return __int_as_float((k + 127) << 23); }

// v * 2^k exactly (the result is far from overflow and underflow), k in [-252, 254]
__device__ __forceinline__ float scale2(float v, int k) {
  if (k > 127) return (v * pow2f(127)) * pow2f(k - 127);
  if (k < -126) return (v * pow2f(-126)) * pow2f(k + 126);
  return v * pow2f(k);
}

// |hi + lo| in units of 2^(E - 49), E = eb - 126, rounded to nearest (within
// one unit), from the floats' bits: no conversions.  eb >= 1 is the largest
// biased exponent of the row's hi parts (subnormals count as exponent 1), so
// the result is at most 2^49.  The parts are taken with four bits more
// (units of 2^(E - 53)) and the sum rounded.
__device__ __forceinline__ uint64_t mag49(float hi, float lo, int eb, uint32_t& neg) {
  const uint32_t bh = __float_as_uint(hi), bl = __float_as_uint(lo);
  const int eh = (bh >> 23) & 0xff, el = (bl >> 23) & 0xff;
  const uint32_t mh = (bh & 0x7fffffu) | (eh ? 0x800000u : 0u);
  const uint32_t ml = (bl & 0x7fffffu) | (el ? 0x800000u : 0u);
  const int sh = max(eh, 1) - eb + 29, sl = max(el, 1) - eb + 29;  // <= 29, resp. <= 5
  const uint64_t uh = sh >= 0 ? (uint64_t)mh << sh : (sh > -24 ? (uint64_t)(mh >> -sh) : 0ull);
  const uint64_t ul = sl >= 0 ? (uint64_t)ml << sl : (sl > -24 ? (uint64_t)(ml >> -sl) : 0ull);
  uint64_t u2;
  if (((bh ^ bl) >> 31) == 0) {
    neg = bh >> 31;
    u2 = uh + ul;
  } else {
    neg = uh >= ul ? bh >> 31 : bl >> 31;
    u2 = uh >= ul ? uh - ul : ul - uh;
  }
  return (u2 + 8) >> 4;
}

// digit s (7 bits, s = 0 most significant) of a magnitude <= 2^49, as the
// bits of the float q (exact: 2^23 + q - 2^23); its upper half is the bf16
__device__ __forceinline__ uint32_t digit_f32(uint64_t u, int s) {
  const uint32_t q = s == 0 ? (uint32_t)(u >> 42) : (uint32_t)(u >> (42 - 7 * s)) & 127u;  // q_0 <= 128
  return __float_as_uint(__fsub_rn(__uint_as_float(0x4B000000u | q), 8388608.0f));
}

__device__ __forceinline__ void cp_async16(void* dst, const void* src) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

// four 8x8 b16 matrices; lane l addresses row (l & 7) of matrix l >> 3
__device__ __forceinline__ void ldsm4(uint32_t r[4], const uint16_t* p) {
  const unsigned a = (unsigned)__cvta_generic_to_shared(p);
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(a)
               : "memory");
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
  for (int i = threadIdx.x; i < kOzN; i += blockDim.x) fx[i] = 1;
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
    uint32_t nr = 0, ni = 0;
    uint64_t ur = 0, ui = 0;
    if (a < Kp) {
      ur = mag49(v.x, v.y, fx[j], nr);
      ui = mag49(v.z, v.w, fx[j], ni);
    }
#pragma unroll
    for (int d = 0; d < kOzDig; ++d) {
      o->hd[d][0][j][a] = (uint16_t)((digit_f32(ur, d) >> 16) | (nr << 15));
      o->hd[d][1][j][a] = (uint16_t)((digit_f32(ui, d) >> 16) | (ni << 15));
    }
  }
  for (int i = threadIdx.x; i < kOzN; i += blockDim.x) o->fx[i] = fx[i];
}

struct OzOut {  // where a sub-tile's results go
  float4* out;
  const int64_t* orow;  // output offset of each row of the sub-tile (-1: none)
  int64_t before;
  int N;
  float4 alpha;
  bool unit;
};

// One warp: rows rb..rb+15 of the sub-tile x columns cb..cb+7, KS k-steps
// of 16.  Each level L = s + u keeps its own exact fp32 sums (re and im; the
// real part takes X_re H_re and (-X_im) H_im in one accumulator, at most
// 2 * 7 * 64 * 127^2 < 2^24).  The loops run digit s of X, k-step, digit u of
// h, so one A fragment serves all u; the seven levels are combined in
// double-float once, then scaled and stored.
template <int KS>
__device__ __forceinline__ void oz_warp_tile(const OzSmem& sm, const int* ex, int rb, int cb, int lane,
                                             const OzOut& o) {
  const int g = lane >> 2, q4 = lane & 3;
  const int arow = (lane & 7) + 8 * ((lane >> 3) & 1), acol = 8 * (lane >> 4);  // A: 16 rows x 16 k
  // B: lanes 0-15 address the real plane, 16-31 the imaginary one (8 columns x 16 k each)
  const int bplane = lane >> 4, bn = lane & 7, bk = 8 * ((lane >> 3) & 1);
  float acc[kOzDig][2][4];
#pragma unroll
  for (int L = 0; L < kOzDig; ++L)
#pragma unroll
    for (int e = 0; e < 4; ++e) acc[L][0][e] = acc[L][1][e] = 0.f;
#pragma unroll
  for (int s = 0; s < kOzDig; ++s) {
#pragma unroll 1
    for (int k = 0; k < KS; ++k) {
      uint32_t xr[4], xi[4], nx[4];
      ldsm4(xr, &sm.xd[s][0][rb + arow][acol + 16 * k]);
      ldsm4(xi, &sm.xd[s][1][rb + arow][acol + 16 * k]);
#pragma unroll
      for (int q = 0; q < 4; ++q) nx[q] = xi[q] ^ 0x80008000u;
#pragma unroll
      for (int u = 0; u < kOzDig - s; ++u) {
        uint32_t hb[4];  // real b0 b1, imaginary b0 b1
        ldsm4(hb, &sm.h.hd[u][bplane][cb + bn][bk + 16 * k]);
        mma_bf16(acc[s + u][0], xr, hb[0], hb[1]);
        mma_bf16(acc[s + u][1], xr, hb[2], hb[3]);
        mma_bf16(acc[s + u][0], nx, hb[2], hb[3]);
        mma_bf16(acc[s + u][1], xi, hb[0], hb[1]);
      }
    }
  }
  // levels -> double-float, scale by 2^(E_r + F_j), times alpha, store
#pragma unroll
  for (int hrow = 0; hrow < 2; ++hrow) {
    const int rl = rb + g + 8 * hrow;
    if (o.orow[rl] < 0) continue;
    float4* orow = o.out + o.orow[rl];
    const int er = ex[rl] - 126;
#pragma unroll
    for (int c = 0; c < 2; ++c) {
      const int e = 2 * hrow + c;
      const int j = cb + 2 * q4 + c;
      if (j >= o.N) continue;
      float h2[2], l2[2];
#pragma unroll
      for (int z = 0; z < 2; ++z) {
        h2[z] = acc[0][z][e] * pow2f(-14);
        l2[z] = 0.f;
#pragma unroll
        for (int L = 1; L < 4; ++L) df_add(h2[z], l2[z], acc[L][z][e] * pow2f(-7 * (L + 2)), 0.f);
        // levels 4-6 lie below 2^-18 of the row scale: their fp32 sum errs
        // by less than 2^-42 of it, the size of the digits' truncation
        // over 64 terms
        df_add(h2[z], l2[z], fmaf(acc[4][z][e], pow2f(-42), fmaf(acc[5][z][e], pow2f(-49), acc[6][z][e] * pow2f(-56))),
               0.f);
      }
      const int sh = er + (sm.h.fx[j] - 126);
      float4 v;
      v.x = scale2(h2[0], sh);
      v.y = scale2(l2[0], sh);
      v.z = scale2(h2[1], sh);
      v.w = scale2(l2[1], sh);
      df_norm(v.x, v.y);
      df_norm(v.z, v.w);
      if (!o.unit) v = DF64::mul(o.alpha, v);
      if (ex[rl] == 255 || sm.h.fx[j] == 255) {  // an Inf or NaN in the row: propagate it
        const float nan = __int_as_float(0x7fffffff);
        v = make_float4(nan, nan, nan, nan);
      }
      orow[o.before * j] = v;
    }
  }
}

__global__ void __launch_bounds__(kOzThreads, 1) k_mp_oz(const MPTask* __restrict__ tasks,
                                                         const int2* __restrict__ tiles, int64_t tile0) {
  extern __shared__ __align__(16) unsigned char oz_raw[];
  OzSmem& sm = *reinterpret_cast<OzSmem*>(oz_raw);
  const int2 tl = tiles[tile0 + blockIdx.x];
  const MPTask t = tasks[tl.x];
  const float4* __restrict__ in = reinterpret_cast<const float4*>(t.in);
  float4* out = reinterpret_cast<float4*>(t.out);
  const int K = t.a_in, N = t.a_out;
  const int Kp = (K + 15) & ~15;
  const int64_t before = t.before;
  const int64_t nrows = before * t.after;
  const int64_t rowA = (int64_t)tl.y * kOzRows * kOzSub;
  const int nsub = (int)min((int64_t)kOzSub, (nrows - rowA + kOzRows - 1) / kOzRows);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

  // h's digits: rows j < N and columns k < Kp of the 14 planes, and h's row exponents
  {
    const unsigned char* src = static_cast<const unsigned char*>(t.oz_h);
    unsigned char* dst = reinterpret_cast<unsigned char*>(&sm.h);
    const int cpr = Kp / 8, per_plane = N * cpr;
    for (int i = tid; i < 2 * kOzDig * per_plane; i += kOzThreads) {
      const int p = i / per_plane, w = i - p * per_plane;
      const int j = w / cpr, c = w - j * cpr;
      const size_t off = ((size_t)p * kOzN + j) * (kOzPitch * 2) + (size_t)c * 16;
      cp_async16(dst + off, src + off);
    }
    const size_t fo = offsetof(OzH, fx);
    for (int i = tid; i < kOzN / 4; i += kOzThreads) cp_async16(dst + fo + 16 * i, src + fo + 16 * i);
  }

  // X of a sub-tile: a thread keeps one row (8 rows x 4 lanes per warp, row
  // groups by warp & 3) and two pairs (a, a + 1) of that row; a warp's
  // 32-bit digit stores then fall in 32 distinct banks
  const int xrow = 8 * (warp & 3) + (lane & 7);
  const int xp0 = (lane >> 3) + 4 * (warp >> 2);  // pairs xp0 + 16 i, i < 2
  float4 xv[kOzPre];
  auto load_x = [&](int sub) {
    const int64_t r = rowA + (int64_t)sub * kOzRows + xrow;
    const bool ok = r < nrows;
    const int64_t b = ok ? r % before : 0, c = ok ? r / before : 0;
    const float4* base = in + b + before * (int64_t)K * c;
    if ((lane >> 3) == 0 && (warp >> 2) == 0) sm.orow[sub & 1][xrow] = ok ? b + before * (int64_t)N * c : -1;
#pragma unroll
    for (int i = 0; i < kOzPre / 2; ++i) {
      const int a = 2 * (xp0 + 16 * i);
      xv[2 * i] = ok && a < K ? base[before * a] : make_float4(0.f, 0.f, 0.f, 0.f);
      xv[2 * i + 1] = ok && a + 1 < K ? base[before * (a + 1)] : make_float4(0.f, 0.f, 0.f, 0.f);
    }
  };

  if (tid < kOzRows) sm.ex[0][tid] = 1;
  load_x(0);
  __syncthreads();

  // warps: two row halves x eight column groups of 8
  const int rb = 16 * (warp & 1), cb = 8 * (warp >> 1);
  const bool active = cb < N;
  OzOut o{out, nullptr, before, N, DF64::coef(t.alpha), t.alpha.x == 1.0 && t.alpha.y == 0.0};

  for (int sub = 0; sub < nsub; ++sub) {
    int* ex = sm.ex[sub & 1];
    // row exponents (the row's four lanes of this warp, then the two warps),
    // then the digits of this sub-tile, all from registers
    {
      int m = 1;
#pragma unroll
      for (int i = 0; i < kOzPre; ++i) m = max(m, max(fexp(xv[i].x), fexp(xv[i].z)));
      m = max(m, __shfl_xor_sync(0xffffffffu, m, 8));
      m = max(m, __shfl_xor_sync(0xffffffffu, m, 16));
      if ((lane >> 3) == 0) atomicMax(&ex[xrow], m);
    }
    __syncthreads();
    {
      const int eb = ex[xrow];
#pragma unroll
      for (int i = 0; i < kOzPre / 2; ++i) {
        const int a = 2 * (xp0 + 16 * i);
        if (a >= Kp) continue;
        uint32_t n0, n1, n2, n3;
        const uint64_t u0 = mag49(xv[2 * i].x, xv[2 * i].y, eb, n0);          // re, a
        const uint64_t u1 = mag49(xv[2 * i + 1].x, xv[2 * i + 1].y, eb, n1);  // re, a + 1
        const uint64_t u2 = mag49(xv[2 * i].z, xv[2 * i].w, eb, n2);          // im, a
        const uint64_t u3 = mag49(xv[2 * i + 1].z, xv[2 * i + 1].w, eb, n3);  // im, a + 1
        const uint32_t sre = (n0 << 15) | (n1 << 31), sim = (n2 << 15) | (n3 << 31);
        uint32_t* pre = reinterpret_cast<uint32_t*>(&sm.xd[0][0][xrow][a]);
        uint32_t* pim = reinterpret_cast<uint32_t*>(&sm.xd[0][1][xrow][a]);
#pragma unroll
        for (int d = 0; d < kOzDig; ++d) {
          pre[d * kOzRows * kOzPitch] = (digit_f32(u0, d) >> 16) | (digit_f32(u1, d) & 0xffff0000u) | sre;
          pim[d * kOzRows * kOzPitch] = (digit_f32(u2, d) >> 16) | (digit_f32(u3, d) & 0xffff0000u) | sim;
        }
      }
    }
    if (tid < kOzRows) sm.ex[(sub + 1) & 1][tid] = 1;
    cp_async_wait_all();
    __syncthreads();
    if (sub + 1 < nsub) load_x(sub + 1);  // in flight during the products

    if (active) {
      o.orow = sm.orow[sub & 1];
      switch (Kp / 16) {
        case 1: oz_warp_tile<1>(sm, ex, rb, cb, lane, o); break;
        case 2: oz_warp_tile<2>(sm, ex, rb, cb, lane, o); break;
        case 3: oz_warp_tile<3>(sm, ex, rb, cb, lane, o); break;
        default: oz_warp_tile<4>(sm, ex, rb, cb, lane, o); break;
      }
    }
    __syncthreads();  // the next sub-tile's digits overwrite xd
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
