// qt_umma.cu -- the contractions of the mixed-precision plans on the
// fifth-generation tensor cores (tcgen05.mma, accumulators in tensor memory).
//
// Double-float plans (QT_PREC_DF64_TC): mode products, hole products and
// last-index accumulations run on one sum-of-products kernel (k_tcs, its
// design above it).  Every operand row is scaled by the power of two 2^-E
// of its largest exponent and cut into seven signed digits by error-free
// splits x_s = fl(fl(r + sigma_s) - sigma_s), sigma_s = 1.5 * 2^(16 - 7s):
// x_s is r rounded to a multiple of 2^(-7(s+1)), r - x_s is exact, the
// value's low word joins from s = 3.  The digit integers
// q_s = x_s 2^(7(s+1)) have |q_s| <= 128, so q_s 2^(-7s) is exact in bf16 and
// every digit product is exact.  Pairs with s + t <= 6 are summed in fp32
// accumulators, one per level L = s + t, as far as tensor memory holds them
// (the last taking the remaining levels together); the epilogue adds the
// levels in double-float and scales by 2^(E_row + F_column).
//
// Complex64 plans (QT_PREC_TF32X3): the mode products as split-TF32 (k_mp_tf):
// X and h (fp32) split into TF32 halves hi + lo; hi*hi + hi*lo + lo*hi
// accumulate in one fp32 sum per output (3 passes).
#include <cuda_runtime.h>

#include <cstdint>

#include "qt_arith.cuh"
#include "qt_internal.h"
#include "qt_tc05.cuh"

namespace qt {
namespace {

using namespace tc05;

constexpr int kRows = 128;                 // rows per tile (M)
constexpr int kDig = 7;                    // digits per value (double-float plans)
constexpr int kThreadsTc = 416;            // thirteen warps (roles per kernel below)
constexpr uint64_t kSpin = 2000000000ull;  // ns before a wait gives up (2 s)
constexpr int kChunkK = 16;                // k per ring stage

// a digit plane of one 16-k step: 128 rows x 16 k bf16 (core layout [kc][g][8][8])
constexpr int kOzAPlane = kRows * kChunkK * 2;        // 4096 bytes
constexpr int kOzAStage = kDig * 2 * kOzAPlane;       // 57344: seven digits, re and im
// TF: a TF32 plane of one stage: 128 rows x 16 k fp32 (core layout [kc][g][8][4])
constexpr int kTfAPlane = kRows * kChunkK * 4;        // 8192 bytes
constexpr int kTfAStage = 4 * kTfAPlane;              // hi_re, hi_im, lo_re, lo_im
constexpr int kTfBMax = 4 * 4 * 64 * 64;              // 65536: K 64, N 64
static_assert(kTfBMax <= kMpOzImageBytes, "operand image slot too small");

struct Bars {
  uint64_t full[2], empty[2], exready[2], exfree[2], tfull, tempty, bfull, drain;
  uint32_t tmem;
  int pad;
};

struct TfSmem {
  unsigned char b[kTfBMax];
  unsigned char a[2][kTfAStage];
  Bars bar;
};
static_assert(sizeof(TfSmem) <= 232448, "shared memory of the split-TF32 kernel exceeds 227 KB");

__device__ __forceinline__ int fexp(float v) { return (__float_as_int(v) >> 23) & 0xff; }
__device__ __forceinline__ float pow2f(int k) { return __int_as_float((k + 127) << 23); }
__device__ __forceinline__ float scale2(float v, int k) {
  if (k > 127) return (v * pow2f(127)) * pow2f(k - 127);
  if (k < -126) return (v * pow2f(-126)) * pow2f(k + 126);
  return v * pow2f(k);
}

// Digits of one double-float value v = hi + lo of a row whose largest biased
// exponent of hi parts is eb (|v| < 2^E, E = eb - 126).  The row is scaled
// to |v 2^-E| < 1 (exactly, by a power of two) and cut by error-free splits
// x_s = fl(fl(r + sigma_s) - sigma_s), sigma_s = 1.5 * 2^(16 - 7s): x_s is r
// rounded to the nearest multiple of 2^(-7(s+1)) and r - x_s is exact, so
// v 2^-E = x_0 + ... + x_6 + (remainder of at most 2^-49).  The low part
// joins from s = 3 (|lo| is below 2^-24 of the row scale); each digit is the
// exact sum of its hi and lo splits.  With q_s = x_s 2^(7(s+1)):
// |q_s| <= 128 -- integers of at most eight significant bits, exact in bf16.
// Stored is x_s itself (bf16), so that a product of digits s and t carries
// its level's weight 2^(-7(s+t+2)).
__device__ __forceinline__ float dsplit(float& r, float sigma) {
  const float x = __fsub_rn(__fadd_rn(r, sigma), sigma);
  r = __fsub_rn(r, x);
  return x;
}
__device__ __forceinline__ float digit_sigma(int s) { return __int_as_float(((127 + 16 - 7 * s) << 23) | 0x400000); }
// v 2^k exactly (row scaling)
__device__ __forceinline__ float row_scale(float v, int k) {
  return (k >= -126 && k <= 127) ? v * pow2f(k) : scale2(v, k);
}
// the seven digits x_s of hi + lo as floats (exact in bf16: their upper
// 16 bits are the bf16)
__device__ __forceinline__ void digits_f32(float hi, float lo, int eb, float d[kDig]) {
  float rh = row_scale(hi, 126 - eb), rl = row_scale(lo, 126 - eb);
#pragma unroll
  for (int s = 0; s < kDig; ++s) {
    float x = dsplit(rh, digit_sigma(s));
    if (s >= 3) x = __fadd_rn(x, dsplit(rl, digit_sigma(s)));
    d[s] = x;
  }
}
// the bf16 of two exact digits in one 32-bit word (a in the low half)
__device__ __forceinline__ uint32_t pack_bf16(float a, float b) {
  return __byte_perm(__float_as_uint(a), __float_as_uint(b), 0x7632);
}

// TF32 halves of x: hi = x rounded to 10 fraction bits, lo = x - hi (the
// tensor core reads the upper 19 bits of each 32-bit operand)
__device__ __forceinline__ void tf32_split(float x, uint32_t& hi, uint32_t& lo) {
  uint32_t h;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(h) : "f"(x));
  hi = h;
  const float r = __fsub_rn(x, __uint_as_float(h));
  uint32_t l;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(l) : "f"(r));
  lo = l;
}

// byte offset, in a K-major core layout of `rows` rows, of row r at the
// 16-byte k-group kc
__device__ __forceinline__ int core_off(int r, int kc, int rows) {
  return kc * (rows / 8) * 128 + (r >> 3) * 128 + (r & 7) * 16;
}

// separate level accumulators that fit tensor memory (512 columns of 2 Np each)
__device__ __forceinline__ int levels_for(int Np) { return min(kDig, 512 / (2 * Np)); }

__device__ __forceinline__ void set_status(int* status, int code) {
  if (status) atomicCAS(status, 0, code);
}

// Write element (j, k) of H^T, value v, into the split-TF32 operand image
// [ks][hi_re, hi_im, lo_re, lo_im][core layout Np x 16 k] fp32.
__device__ __forceinline__ void put_image_tf(unsigned char* img, int Np, int j, int k, float4 v) {
  const int plane_bytes = Np * kChunkK * 4;
  const int ks = k / kChunkK, kk = k % kChunkK;
  const int off = core_off(j, kk / 4, Np) + (kk % 4) * 4;
  unsigned char* base = img + (size_t)ks * 4 * plane_bytes;
  uint32_t hr, lr, hi_, li;
  tf32_split(v.x, hr, lr);
  tf32_split(v.z, hi_, li);
  *reinterpret_cast<uint32_t*>(base + 0 * plane_bytes + off) = hr;
  *reinterpret_cast<uint32_t*>(base + 1 * plane_bytes + off) = hi_;
  *reinterpret_cast<uint32_t*>(base + 2 * plane_bytes + off) = lr;
  *reinterpret_cast<uint32_t*>(base + 3 * plane_bytes + off) = li;
}

// ---------------------------------------------------------------------------
// pre-pass of the split-TF32 mode products: the operand image of alpha h for
// every task of the stage, H^T rows j (N, padded to Np = 16 ceil(N / 16)),
// k < Kp zero-padded
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_mp_tf_h(const MPTask* __restrict__ tasks, const int* __restrict__ ids,
                                                 int64_t first) {
  const MPTask t = tasks[ids[first + blockIdx.x]];
  unsigned char* img = static_cast<unsigned char*>(t.oz_h);
  const float4* __restrict__ h = reinterpret_cast<const float4*>(t.h);
  const int K = t.a_in, N = t.a_out;
  const int Np = (N + 15) & ~15, Kp = (K + 15) & ~15;
  const bool one = t.alpha.x == 1.0 && t.alpha.y == 0.0;
  const float4 cf = C32::coef(t.alpha);
  for (int e = threadIdx.x; e < Np * Kp; e += blockDim.x) {
    const int j = e % Np, k = e / Np;
    float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
    if (j < N && k < K) {
      v = h[j + (int64_t)N * k];
      if (!one) v = C32::mul(cf, v);
    }
    put_image_tf(img, Np, j, k, v);
  }
}

// ---------------------------------------------------------------------------
// One unit of work: 128 rows of a mode-product task.
// ---------------------------------------------------------------------------
struct TcUnit {
  int K, N, Np;              // reduction length, output columns (padded)
  const unsigned char* img;  // h operand image
  int64_t nrows;             // rows of the task
  const float4* in;          // the input tensor
  int64_t before;            // stride of the reduction index
  float4* out;
};

__device__ __forceinline__ TcUnit make_unit(const MPTask* tasks, int task) {
  const MPTask t = tasks[task];
  TcUnit u;
  u.K = t.a_in;
  u.N = t.a_out;
  u.Np = (u.N + 15) & ~15;
  u.img = static_cast<const unsigned char*>(t.oz_h);
  u.nrows = (int64_t)t.before * t.after;
  u.in = reinterpret_cast<const float4*>(t.in);
  u.before = t.before;
  u.out = reinterpret_cast<float4*>(t.out);
  return u;
}

// ---------------------------------------------------------------------------
// Split-TF32 mode products (complex64 plans).  out[b, j, c] =
// alpha sum_a h(j, a) in[b, a, c] is the GEMM Y = X H^T with rows r = (b, c)
// (K = a_in, N = a_out <= 64); four real MMAs per operand pair,
//   Y_re += X_re H_re^T - X_im H_im^T,   Y_im += X_re H_im^T + X_im H_re^T,
// the minus sign by the instruction's negate-A bit.  Roles (416 threads):
// warps 0-7 produce X's TF32 halves of each 16-k step into a two-stage ring
// (two threads per row, eight k each); warp 12 allocates tensor memory, loads
// the h image of the unit (bulk copies, once per change of task) and issues
// the MMAs from one thread; warps 8-11 read the accumulators (warp 8 + q:
// lanes 32q..) and write the outputs.  A CTA takes a contiguous range of
// 128-row tiles.  Every wait is bounded: a wait that runs out sets the status
// word, and the CTA drains its issued MMAs, frees tensor memory and returns.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kThreadsTc, 1) k_mp_tf(const MPTask* __restrict__ tasks,
                                                          const int2* __restrict__ tiles, int64_t tile0,
                                                          int64_t n_tiles, int* status) {
  extern __shared__ __align__(128) unsigned char tc_raw[];
  TfSmem& sm = *reinterpret_cast<TfSmem*>(tc_raw);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int64_t per = n_tiles / gridDim.x, extra = n_tiles % gridDim.x;
  const int64_t my0 = blockIdx.x * per + min((int64_t)blockIdx.x, extra);
  const int64_t my1 = my0 + per + (blockIdx.x < extra ? 1 : 0);

  if (tid == 0) {
    for (int s = 0; s < 2; ++s) {
      mbar_init(&sm.bar.full[s], 256);
      mbar_init(&sm.bar.empty[s], 1);
    }
    mbar_init(&sm.bar.tfull, 1);
    mbar_init(&sm.bar.tempty, 128);
    mbar_init(&sm.bar.bfull, 1);
    mbar_init(&sm.bar.drain, 1);
    mbar_fence_init();
  }
  if (warp == 12) tmem_alloc(&sm.bar.tmem, 128u);
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
  const uint32_t tmem = sm.bar.tmem;
  bool ok = true;

  if (warp < 8) {
    // ---------------- producers: two per row, eight k of every step each ----------------
    const int r = tid & (kRows - 1), h = tid >> 7;
    uint32_t q = 0;
    for (int64_t it = my0; it < my1 && ok; ++it) {
      const int2 tl = tiles[tile0 + it];
      const TcUnit U = make_unit(tasks, tl.x);
      const int K = U.K;
      const int64_t rg = (int64_t)tl.y * kRows + r;
      const bool valid = rg < U.nrows;
      const int64_t b = valid ? rg % U.before : 0, c = valid ? rg / U.before : 0;
      const float4* base = U.in + b + U.before * (int64_t)K * c;
      const int nks = (K + kChunkK - 1) / kChunkK;
      // this thread's eight values of step ks; the next step's loads are in
      // flight while the current one is split
      auto load8 = [&](float4 (&x)[8], int ks) {
#pragma unroll
        for (int i = 0; i < 8; ++i) {
          const int a = ks * kChunkK + h * 8 + i;
          x[i] = (valid && a < K) ? __ldg(base + U.before * a) : make_float4(0.f, 0.f, 0.f, 0.f);
        }
      };
      float4 nx[8];
      load8(nx, 0);
      for (int ks = 0; ks < nks; ++ks, ++q) {
        const int s = q & 1;
        float4 x[8];
#pragma unroll
        for (int i = 0; i < 8; ++i) x[i] = nx[i];
        if (ks + 1 < nks) load8(nx, ks + 1);
        if (!mbar_wait(&sm.bar.empty[s], ((q >> 1) & 1) ^ 1, kSpin)) {
          set_status(status, 1);
          ok = false;
          break;
        }
        unsigned char* A = sm.a[s];
        // fp32 values (complex64 storage keeps them in the hi words)
#pragma unroll
        for (int g2 = 0; g2 < 2; ++g2) {  // two 16-byte core rows of 4 k each
          uint32_t hr[4], hi_[4], lr[4], li[4];
#pragma unroll
          for (int i = 0; i < 4; ++i) {
            tf32_split(x[4 * g2 + i].x, hr[i], lr[i]);
            tf32_split(x[4 * g2 + i].z, hi_[i], li[i]);
          }
          const int off = core_off(r, 2 * h + g2, kRows);
          *reinterpret_cast<uint4*>(A + 0 * kTfAPlane + off) = make_uint4(hr[0], hr[1], hr[2], hr[3]);
          *reinterpret_cast<uint4*>(A + 1 * kTfAPlane + off) = make_uint4(hi_[0], hi_[1], hi_[2], hi_[3]);
          *reinterpret_cast<uint4*>(A + 2 * kTfAPlane + off) = make_uint4(lr[0], lr[1], lr[2], lr[3]);
          *reinterpret_cast<uint4*>(A + 3 * kTfAPlane + off) = make_uint4(li[0], li[1], li[2], li[3]);
        }
        fence_proxy_async();
        mbar_arrive(&sm.bar.full[s]);
      }
    }
  } else if (warp == 12) {
    // ---------------- MMA issue (one thread) and h loads ----------------
    if (lane == 0) {
      uint32_t q = 0, nb = 0, un = 0;
      const void* cur = nullptr;
      for (int64_t it = my0; it < my1 && ok; ++it, ++un) {
        const int2 tl = tiles[tile0 + it];
        const TcUnit U = make_unit(tasks, tl.x);
        const int K = U.K, Np = U.Np, nks = (K + kChunkK - 1) / kChunkK;
        const int plane_b = Np * kChunkK * 4;  // bytes of one h plane per step
        const uint32_t tpar = un & 1;
        if (U.img != cur) {
          // the previous unit's MMAs read the old h: wait until they completed
          if (un > 0 && !mbar_wait(&sm.bar.tfull, tpar ^ 1, kSpin)) {
            set_status(status, 2);
            ok = false;
            break;
          }
          const uint32_t bytes = (uint32_t)(nks * 4 * plane_b);
          mbar_arrive_expect_tx(&sm.bar.bfull, bytes);
          for (uint32_t o = 0; o < bytes; o += 32768u) {
            const uint32_t n = bytes - o < 32768u ? bytes - o : 32768u;
            bulk_g2s(sm.b + o, U.img + o, n, &sm.bar.bfull);
          }
          if (!mbar_wait(&sm.bar.bfull, nb & 1, kSpin)) {
            set_status(status, 3);
            ok = false;
            break;
          }
          ++nb;
          cur = U.img;
        }
        // the epilogue released the accumulators of the previous unit
        if (!mbar_wait(&sm.bar.tempty, tpar ^ 1, kSpin)) {
          set_status(status, 4);
          ok = false;
          break;
        }
        fence_after_sync();
        const uint32_t lboB = (uint32_t)(Np / 8) * 128;
        const uint32_t lboA4 = (kRows / 8) * 128;  // kc stride of a 16-k fp32 plane: [kc (4)][g][8][4]
        const uint32_t id = idesc_m128(2, Np, false), idn = idesc_m128(2, Np, true);
        uint32_t used = 0;  // 0 until the unit's first MMAs
        for (int ks = 0; ks < nks; ++ks, ++q) {
          const int s = q & 1;
          if (!mbar_wait(&sm.bar.full[s], (q >> 1) & 1, kSpin)) {
            set_status(status, 5);
            ok = false;
            break;
          }
          fence_after_sync();
          const uint32_t a0 = smem_u32(sm.a[s]);
          const uint32_t b0 = smem_u32(sm.b) + (uint32_t)(ks * 4 * plane_b);
#pragma unroll 1
          for (int h8 = 0; h8 < 2; ++h8) {  // two MMAs of k = 8 per step
            const uint32_t ao = (uint32_t)(2 * h8) * lboA4, bo = (uint32_t)(2 * h8) * lboB;
            const uint64_t ahr = desc_kmajor(a0 + 0 * kTfAPlane + ao, lboA4, 128);
            const uint64_t ahi = desc_kmajor(a0 + 1 * kTfAPlane + ao, lboA4, 128);
            const uint64_t alr = desc_kmajor(a0 + 2 * kTfAPlane + ao, lboA4, 128);
            const uint64_t ali = desc_kmajor(a0 + 3 * kTfAPlane + ao, lboA4, 128);
            const uint64_t bhr = desc_kmajor(b0 + 0 * plane_b + bo, lboB, 128);
            const uint64_t bhi = desc_kmajor(b0 + 1 * plane_b + bo, lboB, 128);
            const uint64_t blr = desc_kmajor(b0 + 2 * plane_b + bo, lboB, 128);
            const uint64_t bli = desc_kmajor(b0 + 3 * plane_b + bo, lboB, 128);
            const uint32_t dre = tmem, dim_ = tmem + (uint32_t)Np;
            const uint32_t f = used;  // 0 only for the first MMAs of the unit
            // lo x hi and hi x lo first, then hi x hi
            mma_tf32(dre, alr, bhr, id, f);
            mma_tf32(dim_, alr, bhi, id, f);
            mma_tf32(dre, ali, bhi, idn, 1);
            mma_tf32(dim_, ali, bhr, id, 1);
            mma_tf32(dre, ahr, blr, id, 1);
            mma_tf32(dim_, ahr, bli, id, 1);
            mma_tf32(dre, ahi, bli, idn, 1);
            mma_tf32(dim_, ahi, blr, id, 1);
            mma_tf32(dre, ahr, bhr, id, 1);
            mma_tf32(dim_, ahr, bhi, id, 1);
            mma_tf32(dre, ahi, bhi, idn, 1);
            mma_tf32(dim_, ahi, bhr, id, 1);
            used = 1;
          }
          commit(&sm.bar.empty[s]);  // the step is free once these MMAs completed
        }
        if (!ok) break;
        commit(&sm.bar.tfull);
      }
      // drain: every MMA issued by this thread completed before tensor memory is freed
      commit(&sm.bar.drain);
      if (!mbar_wait(&sm.bar.drain, 0, kSpin)) set_status(status, 6);
    }
  } else {
    // ---------------- epilogue: warp 8 + qd reads lanes 32 qd .. ----------------
    const int qd = warp - 8;
    const int r = 32 * qd + lane;
    const uint32_t lane_addr = tmem + ((uint32_t)(32 * qd) << 16);
    uint32_t un = 0;
    for (int64_t it = my0; it < my1 && ok; ++it, ++un) {
      const int2 tl = tiles[tile0 + it];
      const TcUnit U = make_unit(tasks, tl.x);
      const int N = U.N, Np = U.Np;
      if (!mbar_wait(&sm.bar.tfull, un & 1, kSpin)) {
        set_status(status, 7);
        ok = false;
        break;
      }
      fence_after_sync();
      const int64_t rg = (int64_t)tl.y * kRows + r;
      const bool live = rg < U.nrows;
      const int64_t ro = live ? rg % U.before + U.before * (int64_t)N * (rg / U.before) : 0;
      for (int j0 = 0; j0 < Np; j0 += 8) {
        __syncwarp();  // the tensor-memory loads below are warp-collective
        float vre[8], vim[8];
        tmem_ld8(lane_addr + (uint32_t)j0, vre);
        tmem_ld8(lane_addr + (uint32_t)(Np + j0), vim);
        tmem_wait_ld();
#pragma unroll
        for (int i = 0; i < 8; ++i) {
          const int j = j0 + i;
          if (live && j < N) U.out[ro + U.before * j] = make_float4(vre[i], 0.f, vim[i], 0.f);
        }
      }
      fence_before_sync();
      mbar_arrive(&sm.bar.tempty);
    }
  }
  fence_before_sync();
  __syncthreads();
  if (warp == 12) {
    fence_after_sync();
    tmem_dealloc(tmem, 128u);
  }
}

// ---------------------------------------------------------------------------
// Sums of products on the tensor cores (double-float plans): the hole
// products and the last-index accumulations.  Both compute, per output row
// m and column n,
//   D(m, n) = sum over units u of  sum_k X_u(m, k) W_u(n, k)     (complex)
// in units of at most 64 k, every unit with its own power-of-two scales per
// row of X_u (E_m) and per row of W_u (F_n):
//  * hole products S_t(i, j) = sum_k conj(A[k; i]) B_t[k; j]: the rows m are
//    the (task t, j) of a group of tasks that share A (X = B_t), n = i and
//    W = conj(A); the units are the 64-k chunks of the reduction;
//  * accumulations out[r, j] (+)= alpha sum_t sum_j' H_t(j, j') X_t[r, j']:
//    rows m = r (a block of 128), n = j, one unit per term t with X = X_t
//    and W = alpha H_t (alpha I for identity terms).
// The accumulator tile has 2 np columns, the real parts for n < np and the
// imaginary parts after them, so
//   Re D = Xr Wr - Xi Wi,   Im D = Xr Wi + Xi Wr
// are two MMAs of N = 2 np per digit pair: Xr x [Wr | Wi] and
// Xi x [-Wi | Wr].  W's image, written by a pre-pass per unit, stores the
// rows [-Wi | Wr | Wi] (np each) once per 16-k step and digit; the two
// operands are its rows np.. and 0.. .  The producers cut X's digits; the
// image steps arrive by bulk copies on the same barrier.  A unit's level
// sums are exact in fp32 (at most 7 pairs x 2 x 64 products of |digit
// products| <= 2^14 units per level); the epilogue recombines them in
// double-float, scales by 2^(E_m + F_n) and adds them to the output in
// double-float (a work item's first unit stores, or adds to the old output
// where the accumulation asks for it).
// ---------------------------------------------------------------------------
constexpr int kTcsNStage = kDig * 3 * 64 * 32;  // W side of one 16-k step at np = 64

enum { TCS_HP = 0, TCS_ACC = 1, TCS_MP = 2 };

struct TcsSmem {
  unsigned char a[2][kOzAStage];
  unsigned char n[2][kTcsNStage];
  Bars bar;
  uint8_t ex[2][kRows];  // the row exponents of the two units in flight
  int fx[8][64];         // the unit's column exponents, one copy per epilogue warp
};
static_assert(sizeof(TcsSmem) <= 232448, "shared memory of the sum-of-products kernel exceeds 227 KB");

struct TcsArgs {
  const HPTask* hp;          // hole products: tasks, groups, partial tiles
  const HpTcGroup* groups;
  double2* ws;
  const AccTask* acc;        // accumulations: tasks and terms
  const AccTerm* terms;
  const MPTask* mp;          // mode products: tasks, tiles (task, 128-row block) and the pre-pass's tasks
  const int2* mp_tiles;
  const int* mp_tasks;
  const int4* items;         // HP (group, range z, first chunk, end chunk); ACC (task, block, units before, 0)
  int64_t item0, n_items;
  int64_t units;             // ACC: units of all items (weighted split over the CTAs)
  int* status;
};

// item `it` of the launch (mode products: (task, 128-row block, 0, 0))
template <int OP>
__device__ __forceinline__ int4 tcs_fetch(const TcsArgs& g, int64_t it) {
  if (OP == TCS_MP) {
    const int2 t = g.mp_tiles[g.item0 + it];
    return make_int4(t.x, t.y, 0, 0);
  }
  return g.items[g.item0 + it];
}

// element k of row `row` of a hole-product operand of shape (before, a, after):
// k = b + before c, offset b + before row + before a c; walked in steps of one
struct KWalk {
  int b, c;
  __device__ __forceinline__ KWalk(int k, int before) : b(k - (k / before) * before), c(k / before) {}
  __device__ __forceinline__ int64_t off(int row, int before, int a) const {
    return b + (int64_t)before * row + (int64_t)before * a * c;
  }
  __device__ __forceinline__ void next(int before) {
    if (++b == before) {
      b = 0;
      ++c;
    }
  }
};

// the CTA's run of items: equal counts (HP: items of about equal length), or
// the items whose first unit falls into the CTA's equal share of all units
template <int OP>
__device__ __forceinline__ void tcs_range(const TcsArgs& g, int64_t& i0, int64_t& i1) {
  if (OP != TCS_ACC) {
    const int64_t per = g.n_items / gridDim.x, extra = g.n_items % gridDim.x;
    i0 = blockIdx.x * per + min((int64_t)blockIdx.x, extra);
    i1 = i0 + per + (blockIdx.x < extra ? 1 : 0);
    return;
  }
  auto first_at = [&](int64_t u) {  // first item with units-before >= u
    int64_t lo = 0, hi = g.n_items;
    while (lo < hi) {
      const int64_t mid = (lo + hi) >> 1;
      if ((int64_t)g.items[g.item0 + mid].z < u) lo = mid + 1;
      else hi = mid;
    }
    return lo;
  };
  i0 = first_at(g.units * blockIdx.x / gridDim.x);
  i1 = first_at(g.units * (blockIdx.x + 1) / gridDim.x);
}

// per item: padded columns np, real columns, units, 16-k steps per unit
struct TcsItem {
  int np, ncols, nunits, nks;
  int nl;  // level accumulators
};
template <int OP>
__device__ __forceinline__ TcsItem tcs_item(const TcsArgs& g, int4 itm) {
  TcsItem v;
  if (OP == TCS_HP) {
    const HpTcGroup& G = g.groups[itm.x];
    v.np = G.ap;
    v.ncols = G.a;
    v.nunits = itm.w - itm.z;
    v.nks = hp_tc_kc(G.ap) / kChunkK;
    // 128-k chunks keep four accumulators (levels 0..2 exact up to 170 k)
    v.nl = v.nks > 4 ? min(4, levels_for(G.ap)) : levels_for(G.ap);
  } else if (OP == TCS_ACC) {
    const AccTask& T = g.acc[itm.x];
    v.np = (T.d + 7) & ~7;
    v.ncols = T.d;
    v.nunits = T.count;
    v.nks = (T.d + kChunkK - 1) / kChunkK;
    v.nl = levels_for(v.np);
  } else {
    const MPTask& t = g.mp[itm.x];
    v.np = (t.a_out + 7) & ~7;
    v.ncols = t.a_out;
    v.nunits = 1;
    v.nks = (t.a_in + kChunkK - 1) / kChunkK;
    v.nl = levels_for(v.np);
  }
  return v;
}
// image steps of a unit (the image's layout; the unit may use fewer)
template <int OP>
__device__ __forceinline__ int tcs_img_steps(int np) {
  return OP == TCS_HP ? hp_tc_kc(np) / kChunkK : 4;
}
template <int OP>
__device__ __forceinline__ const unsigned char* tcs_image(const TcsArgs& g, int4 itm, int u, int np) {
  const int64_t cb = hp_tc_chunk_bytes(np, tcs_img_steps<OP>(np));
  if (OP == TCS_HP) return g.groups[itm.x].img + (size_t)(itm.z + u) * cb;
  if (OP == TCS_MP) return static_cast<const unsigned char*>(g.mp[itm.x].oz_h);
  return static_cast<const unsigned char*>(g.acc[itm.x].tc_img) + (size_t)u * cb;
}

// pre-pass: the image of W for one unit -- per 16-k step and digit a plane of
// 3 np rows, -Wi at row n, Wr at np + n, Wi at 2 np + n (rows past the last
// column zero) -- and the unit's row exponents F_n.  Thread (n, q) takes row
// n of the steps q, q + 4, ...  HP units (group, chunk): W(i, k) = conj(A[k; i]);
// ACC units (task, term): W(j, k) = alpha H(j, k), alpha I for identity terms;
// MP units (task): W(j, k) = alpha h(j, k).
template <int OP>
__global__ void __launch_bounds__(256) k_tcs_img(TcsArgs g, const int2* __restrict__ units, int64_t first) {
  const int2 u = OP == TCS_MP ? make_int2(g.mp_tasks[first + blockIdx.x], 0) : units[first + blockIdx.x];
  const int n = threadIdx.x & 63, q = threadIdx.x >> 6;
  int np, ncols, steps;
  unsigned char* img;
  // the 16 values of row n at step ks
  auto load16 = [&](int ks, float4 (&v)[16]) {
    if (OP == TCS_HP) {
      const HpTcGroup& G = g.groups[u.x];
      const int K = G.before * G.after, k0 = u.y * hp_tc_kc(G.ap) + ks * kChunkK;
      const float4* __restrict__ A = reinterpret_cast<const float4*>(G.A);
      KWalk w(min(k0, K), G.before);
#pragma unroll
      for (int kk = 0; kk < 16; ++kk) {
        float4 x = make_float4(0.f, 0.f, 0.f, 0.f);
        if (n < G.a && k0 + kk < K) {
          x = __ldg(A + w.off(n, G.before, G.a));
          x.z = -x.z;
          x.w = -x.w;
        }
        v[kk] = x;
        w.next(G.before);
      }
    } else if (OP == TCS_MP) {
      const MPTask& t = g.mp[u.x];
      const float4 cf = DF64::coef(t.alpha);
      const bool one = t.alpha.x == 1.0 && t.alpha.y == 0.0;
      const float4* __restrict__ H = reinterpret_cast<const float4*>(t.h);
#pragma unroll
      for (int kk = 0; kk < 16; ++kk) {
        const int k = ks * kChunkK + kk;
        float4 x = make_float4(0.f, 0.f, 0.f, 0.f);
        if (n < t.a_out && k < t.a_in) {
          x = __ldg(H + n + (int64_t)t.a_out * k);
          if (!one) x = DF64::mul(cf, x);
        }
        v[kk] = x;
      }
    } else {
      const AccTask& T = g.acc[u.x];
      const AccTerm tm = g.terms[T.first + u.y];
      const double2 alpha = T.alpha_ptr ? *T.alpha_ptr : T.alpha;
      const float4 cf = DF64::coef(alpha);
      const float4* __restrict__ H = reinterpret_cast<const float4*>(tm.H);
#pragma unroll
      for (int kk = 0; kk < 16; ++kk) {
        const int k = ks * kChunkK + kk;
        float4 x = make_float4(0.f, 0.f, 0.f, 0.f);
        if (n < T.d && k < T.d) {
          if (H) x = DF64::mul(cf, __ldg(H + n + (int64_t)T.d * k));
          else if (n == k) x = cf;
        }
        v[kk] = x;
      }
    }
  };
  if (OP == TCS_HP) {
    const HpTcGroup& G = g.groups[u.x];
    np = G.ap;
    ncols = G.a;
    steps = hp_tc_kc(np) / kChunkK;
    img = G.img + (size_t)u.y * hp_tc_chunk_bytes(np, steps);
  } else if (OP == TCS_MP) {
    const MPTask& t = g.mp[u.x];
    np = (t.a_out + 7) & ~7;
    ncols = t.a_out;
    steps = 4;
    img = static_cast<unsigned char*>(t.oz_h);
  } else {
    const AccTask& T = g.acc[u.x];
    np = (T.d + 7) & ~7;
    ncols = T.d;
    steps = 4;
    img = static_cast<unsigned char*>(T.tc_img) + (size_t)u.y * hp_tc_chunk_bytes(np, steps);
  }
  (void)ncols;
  __shared__ int fx[64];
  if (threadIdx.x < 64) fx[threadIdx.x] = 1;
  __syncthreads();
  int m = 1;
  for (int ks = q; ks < steps; ks += 4) {
    float4 v[16];
    load16(ks, v);
#pragma unroll
    for (int kk = 0; kk < 16; ++kk) m = max(m, max(fexp(v[kk].x), fexp(v[kk].z)));
  }
  atomicMax(&fx[n], m);
  __syncthreads();
  if (n < np) {
    const int f = fx[n];
    const int rows = 3 * np, plane = rows * 32;
    for (int ks = q; ks < steps; ks += 4) {
      float4 v[16];
      load16(ks, v);
      unsigned char* base = img + (size_t)ks * kDig * plane;
#pragma unroll
      for (int c = 0; c < 2; ++c) {  // the two 8-k core rows of the step
        uint32_t wr[kDig][4], wi[kDig][4];
#pragma unroll
        for (int p = 0; p < 4; ++p) {
          float d0[kDig], d1[kDig], e0[kDig], e1[kDig];
          digits_f32(v[8 * c + 2 * p].x, v[8 * c + 2 * p].y, f, d0);
          digits_f32(v[8 * c + 2 * p + 1].x, v[8 * c + 2 * p + 1].y, f, d1);
          digits_f32(v[8 * c + 2 * p].z, v[8 * c + 2 * p].w, f, e0);
          digits_f32(v[8 * c + 2 * p + 1].z, v[8 * c + 2 * p + 1].w, f, e1);
#pragma unroll
          for (int d = 0; d < kDig; ++d) {
            wr[d][p] = pack_bf16(d0[d], d1[d]);
            wi[d][p] = pack_bf16(e0[d], e1[d]);
          }
        }
#pragma unroll
        for (int d = 0; d < kDig; ++d) {
          unsigned char* pl = base + (size_t)d * plane;
          const uint4 re = make_uint4(wr[d][0], wr[d][1], wr[d][2], wr[d][3]);
          const uint4 im = make_uint4(wi[d][0], wi[d][1], wi[d][2], wi[d][3]);
          const uint4 nim =
              make_uint4(im.x ^ 0x80008000u, im.y ^ 0x80008000u, im.z ^ 0x80008000u, im.w ^ 0x80008000u);
          *reinterpret_cast<uint4*>(pl + core_off(n, c, rows)) = nim;
          *reinterpret_cast<uint4*>(pl + core_off(np + n, c, rows)) = re;
          *reinterpret_cast<uint4*>(pl + core_off(2 * np + n, c, rows)) = im;
        }
      }
    }
  }
  if (threadIdx.x < 64) reinterpret_cast<int*>(img + (size_t)steps * kDig * 3 * np * 32)[threadIdx.x] = fx[threadIdx.x];
}

// pre-pass of the hole products: the biased row exponents E of the M side
// (the members' B rows j, 128 per item) over the item's chunk, into the
// group's table, so that the producers need not read every row twice.  Block
// (item, q) takes the rows 32 q .. 32 q + 31.  With before > 1 a row's k are
// contiguous in memory: a warp takes four rows at once, its lanes along k;
// with before == 1 consecutive rows are: lane l takes row 32 q + l, the
// eight warps an eighth of the chunk each.
__global__ void __launch_bounds__(256) k_hp_ex(TcsArgs g) {
  const int4 itm = g.items[g.item0 + blockIdx.x];
  const HpTcGroup& G = g.groups[itm.x];
  const int before = G.before, a = G.a, K = before * G.after, kc = hp_tc_kc(G.ap);
  const int k0 = itm.z * kc, k1 = min(K, k0 + kc);
  const int rows = G.n * a, m0 = 32 * (int)blockIdx.y;
  unsigned char* ex = G.ex + (size_t)itm.z * kRows;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (before > 1) {
    int e[4];
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      const int m = m0 + warp + 8 * r;
      e[r] = 1;
      if (m < rows) {
        const int mi = m / a, j = m - mi * a;
        const float4* __restrict__ B = reinterpret_cast<const float4*>(g.hp[G.member[mi]].B);
#pragma unroll
        for (int s = 0; s < 4; ++s) {  // kc <= 128: four k per lane
          const int k = k0 + lane + 32 * s;
          if (k < k1) {
            const int c = k / before, b = k - c * before;
            const float4 x = __ldg(B + b + (int64_t)before * j + (int64_t)before * a * c);
            e[r] = max(e[r], max(fexp(x.x), fexp(x.z)));
          }
        }
      }
    }
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      int v = e[r];
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
      if (lane == 0) ex[m0 + warp + 8 * r] = (uint8_t)v;
    }
  } else {
    __shared__ int part[8][32];
    const int m = m0 + lane;
    int e = 1;
    if (m < rows) {
      const int mi = m / a, j = m - mi * a;
      const float4* __restrict__ B = reinterpret_cast<const float4*>(g.hp[G.member[mi]].B);
      const int span = (k1 - k0 + 7) >> 3;
      const int ka = k0 + warp * span, kb = min(k1, ka + span);
      for (int k = ka; k < kb; ++k) {
        const float4 x = __ldg(B + j + (int64_t)a * k);
        e = max(e, max(fexp(x.x), fexp(x.z)));
      }
    }
    part[warp][lane] = e;
    __syncthreads();
    if (warp == 0) {
      int v = part[0][lane];
#pragma unroll
      for (int w = 1; w < 8; ++w) v = max(v, part[w][lane]);
      ex[m] = (uint8_t)v;
    }
  }
}

// the producers' view of row r of an item: its source of X and validity
struct TcsRow {
  bool valid;
  const float4* src;  // HP: B_t; ACC: unused (the term's X)
  int64_t rg;         // ACC: row of the task
  int j;              // HP: column of S_t
};

// Roles (416 threads): warps 0-3 produce X's digits, one thread per row of
// the tile (each 16-k step in two halves of eight k; first the row's
// exponent over the unit's k, then the digits step by step, the next half's
// loads in flight); warp 4 allocates tensor memory and issues the MMAs from
// one thread; warps 5-12 read the accumulators and update the outputs,
// warp w reading lanes 32 (w % 4).. (tensor memory's lane quarter of its
// sub-partition) for half (w - 5) / 4 of the columns.  Every wait is bounded:
// a wait that runs out sets the status word, and the CTA drains its issued
// MMAs, frees tensor memory and returns.
constexpr int kTcsProducers = 128, kTcsEpilogue = 256;
template <int OP>
__global__ void __launch_bounds__(kThreadsTc, 1) k_tcs(TcsArgs g) {
  extern __shared__ __align__(128) unsigned char tcs_raw[];
  TcsSmem& sm = *reinterpret_cast<TcsSmem*>(tcs_raw);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  int64_t my0, my1;
  tcs_range<OP>(g, my0, my1);
  int* status = g.status;

  if (tid == 0) {
    for (int s = 0; s < 2; ++s) {
      mbar_init(&sm.bar.full[s], kTcsProducers);
      mbar_init(&sm.bar.empty[s], 1);
      mbar_init(&sm.bar.exready[s], kTcsProducers);
      mbar_init(&sm.bar.exfree[s], kTcsEpilogue);
    }
    mbar_init(&sm.bar.tfull, 1);
    mbar_init(&sm.bar.tempty, kTcsEpilogue);
    mbar_init(&sm.bar.drain, 1);
    mbar_fence_init();
  }
  if (warp == 4) tmem_alloc(&sm.bar.tmem, 512u);
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
  const uint32_t tmem = sm.bar.tmem;
  bool ok = true;

  if (warp < 4) {
    // ---------------- producers: one per row ----------------
    const int r = tid;
    uint32_t q = 0, un = 0;
    for (int64_t it = my0; it < my1 && ok; ++it) {
      const int4 itm = tcs_fetch<OP>(g, it);
      const TcsItem I = tcs_item<OP>(g, itm);
      const uint32_t nbytes = (uint32_t)(kDig * 3 * I.np * 32);
      // row r of the item
      TcsRow R;
      int before = 1, a = 1, K = 0;
      int64_t rows = 0;  // k stride of X (ACC: the task's rows; MP: before)
      int tfirst = 0;
      if (OP == TCS_HP) {
        const HpTcGroup& G = g.groups[itm.x];
        before = G.before;
        a = G.a;
        K = before * G.after;
        const int mi = r / a;
        R.j = r - mi * a;
        R.valid = mi < G.n;
        R.src = R.valid ? reinterpret_cast<const float4*>(g.hp[G.member[mi]].B) : nullptr;
        R.rg = 0;
      } else if (OP == TCS_ACC) {
        const AccTask& T = g.acc[itm.x];
        rows = T.rows;
        K = T.d;
        tfirst = T.first;
        R.rg = (int64_t)itm.y * kRows + r;
        R.valid = R.rg < rows;
        R.src = nullptr;
        R.j = 0;
      } else {
        // mode product: row (b, c) of the input, its k-th element at b + before (k + a_in c)
        const MPTask& t = g.mp[itm.x];
        const int64_t rg = (int64_t)itm.y * kRows + r;
        K = t.a_in;
        rows = t.before;
        R.valid = rg < (int64_t)t.before * t.after;
        const int64_t b = R.valid ? rg % t.before : 0, c = R.valid ? rg / t.before : 0;
        R.src = reinterpret_cast<const float4*>(t.in) + b + (int64_t)t.before * K * c;
        R.rg = 0;
        R.j = 0;
      }
      for (int u = 0; u < I.nunits; ++u, ++un) {
        const int buf = (int)(un & 1);
        const uint32_t use_par = (un >> 1) & 1;
        const float4* X = OP != TCS_ACC ? R.src : reinterpret_cast<const float4*>(g.terms[tfirst + u].X) + R.rg;
        const int kbase = OP == TCS_HP ? (itm.z + u) * I.nks * kChunkK : 0;
        // the eight values of half hh of step ks: k = kbase + 16 ks + 8 hh + i
        auto load8 = [&](float4 (&x)[8], int ks, int hh) {
          const int k0 = kbase + ks * kChunkK + hh * 8;
          if (OP == TCS_HP) {
            KWalk w(min(k0, K), before);
#pragma unroll
            for (int i = 0; i < 8; ++i) {
              x[i] = (R.valid && k0 + i < K) ? __ldg(X + w.off(R.j, before, a)) : make_float4(0.f, 0.f, 0.f, 0.f);
              w.next(before);
            }
          } else {
#pragma unroll
            for (int i = 0; i < 8; ++i)
              x[i] = (R.valid && k0 + i < K) ? __ldg(X + rows * (k0 + i)) : make_float4(0.f, 0.f, 0.f, 0.f);
          }
        };
        // the row's largest exponent over the unit's k (hole products: from
        // the pre-pass), eight loads in flight
        int eb = 1;
        if (OP == TCS_HP)
          eb = g.groups[itm.x].ex[(size_t)(itm.z + u) * kRows + r];
        else if (R.valid)
          for (int h8 = 0; h8 < 2 * I.nks; ++h8) {
            float4 x[8];
            load8(x, h8 >> 1, h8 & 1);
#pragma unroll
            for (int i = 0; i < 8; ++i) eb = max(eb, max(fexp(x[i].x), fexp(x[i].z)));
          }
        // the epilogue of the unit two back has read ex of this buffer
        if (!mbar_wait(&sm.bar.exfree[buf], use_par ^ 1, kSpin)) {
          set_status(status, 18);
          ok = false;
          break;
        }
        sm.ex[buf][r] = (uint8_t)eb;
        mbar_arrive(&sm.bar.exready[buf]);
        const unsigned char* img = tcs_image<OP>(g, itm, u, I.np);
        float4 nx[8];
        load8(nx, 0, 0);
        for (int ks = 0; ks < I.nks; ++ks, ++q) {
          const int s = q & 1;
          if (!mbar_wait(&sm.bar.empty[s], ((q >> 1) & 1) ^ 1, kSpin)) {
            set_status(status, 11);
            ok = false;
            break;
          }
          if (tid == 0) {
            // W's digits of this step; the copy completes on full[s] (it
            // finishes within microseconds, before any wait could run out)
            mbar_expect_tx(&sm.bar.full[s], nbytes);
            bulk_g2s(sm.n[s], img + (size_t)ks * nbytes, nbytes, &sm.bar.full[s]);
          }
          unsigned char* As = sm.a[s];
#pragma unroll 1
          for (int hh = 0; hh < 2; ++hh) {
            float4 x[8];
#pragma unroll
            for (int i = 0; i < 8; ++i) x[i] = nx[i];
            const int nk = ks + hh;  // the next half: (ks, 1) or (ks + 1, 0)
            if (nk < I.nks) load8(nx, nk, hh ^ 1);
            uint32_t wr[kDig][4], wi[kDig][4];
#pragma unroll
            for (int i = 0; i < 4; ++i) {
              float d0[kDig], d1[kDig], e0[kDig], e1[kDig];
              digits_f32(x[2 * i].x, x[2 * i].y, eb, d0);
              digits_f32(x[2 * i + 1].x, x[2 * i + 1].y, eb, d1);
              digits_f32(x[2 * i].z, x[2 * i].w, eb, e0);
              digits_f32(x[2 * i + 1].z, x[2 * i + 1].w, eb, e1);
#pragma unroll
              for (int d = 0; d < kDig; ++d) {
                wr[d][i] = pack_bf16(d0[d], d1[d]);
                wi[d][i] = pack_bf16(e0[d], e1[d]);
              }
            }
            const int off = core_off(r, hh, kRows);
#pragma unroll
            for (int d = 0; d < kDig; ++d) {
              *reinterpret_cast<uint4*>(As + (2 * d + 0) * kOzAPlane + off) =
                  make_uint4(wr[d][0], wr[d][1], wr[d][2], wr[d][3]);
              *reinterpret_cast<uint4*>(As + (2 * d + 1) * kOzAPlane + off) =
                  make_uint4(wi[d][0], wi[d][1], wi[d][2], wi[d][3]);
            }
          }
          fence_proxy_async();
          mbar_arrive(&sm.bar.full[s]);
        }
        if (!ok) break;
      }
    }
  } else if (warp == 4) {
    // ---------------- MMA issue (one thread) ----------------
    if (lane == 0) {
      uint32_t q = 0, un = 0;
      for (int64_t it = my0; it < my1 && ok; ++it) {
        const int4 itm = tcs_fetch<OP>(g, it);
        const TcsItem I = tcs_item<OP>(g, itm);
        const int np = I.np, NL = I.nl;
        const uint32_t id = idesc_m128(1, 2 * np, false);
        const uint32_t lboA = (kRows / 8) * 128, lboN = (uint32_t)(3 * np / 8) * 128;
        const uint64_t pA = kOzAPlane >> 4, pN = (uint64_t)((3 * np * 32) >> 4);
        const uint64_t p1 = (uint64_t)((np / 8) * 128 >> 4);  // rows np..: [Wr | Wi]
        for (int u = 0; u < I.nunits && ok; ++u, ++un) {
          if (!mbar_wait(&sm.bar.tempty, (un & 1) ^ 1, kSpin)) {
            set_status(status, 14);
            ok = false;
            break;
          }
          fence_after_sync();
          for (int ks = 0; ks < I.nks; ++ks, ++q) {
            const int s = q & 1;
            if (!mbar_wait(&sm.bar.full[s], (q >> 1) & 1, kSpin)) {
              set_status(status, 15);
              ok = false;
              break;
            }
            fence_after_sync();
            const uint64_t dA = desc_kmajor(smem_u32(sm.a[s]), lboA, 128);
            const uint64_t dN = desc_kmajor(smem_u32(sm.n[s]), lboN, 128);
            const uint32_t first = ks == 0 ? 1u : 0u;
#pragma unroll
            for (int sd = 0; sd < kDig; ++sd) {
              const uint64_t ar = dA + (uint64_t)(2 * sd) * pA, ai = ar + pA;
#pragma unroll
              for (int td = 0; td + sd < kDig; ++td) {
                const int L = sd + td < NL - 1 ? sd + td : NL - 1;
                const uint64_t nb = dN + (uint64_t)td * pN;
                const uint32_t d = tmem + (uint32_t)(L * 2 * np);
                const uint32_t acc = (first && sd == 0 && td == L) ? 0u : 1u;
                mma_bf16(d, ar, nb + p1, id, acc);  // Xr x [Wr | Wi]
                mma_bf16(d, ai, nb, id, 1);         // Xi x [-Wi | Wr]
              }
            }
            commit(&sm.bar.empty[s]);
          }
          if (!ok) break;
          commit(&sm.bar.tfull);
        }
      }
      commit(&sm.bar.drain);
      if (!mbar_wait(&sm.bar.drain, 0, kSpin)) set_status(status, 16);
    }
  } else {
    // ---------------- epilogue: warps 5..12, lane quarter w % 4, column half (w - 5) / 4 ----------------
    const int qd = warp & 3, half = (warp - 5) >> 2;
    const int r = 32 * qd + lane;
    const uint32_t lane_addr = tmem + ((uint32_t)(32 * qd) << 16);
    int* fxw = sm.fx[warp - 5];
    uint32_t un = 0;
    for (int64_t it = my0; it < my1 && ok; ++it) {
      const int4 itm = tcs_fetch<OP>(g, it);
      const TcsItem I = tcs_item<OP>(g, itm);
      const int np = I.np, NL = I.nl;
      const int c0 = half * (np >> 1), c1 = c0 + (np >> 1);  // this warp's columns
      // output row r: element n at base[n * stride]
      float4* base = nullptr;
      int64_t stride = 1;
      bool add_first = false;
      if (OP == TCS_HP) {
        const HpTcGroup& G = g.groups[itm.x];
        const int mi = r / G.a, j = r - mi * G.a;
        if (mi < G.n) {
          const HPTask& t = g.hp[G.member[mi]];
          double2* dst = t.splits <= 1 ? t.S : g.ws + t.ws + (int64_t)itm.y * G.a * G.a;
          base = reinterpret_cast<float4*>(dst) + (int64_t)G.a * j;
        }
      } else if (OP == TCS_ACC) {
        const AccTask& T = g.acc[itm.x];
        const int64_t rg = (int64_t)itm.y * kRows + r;
        if (rg < T.rows) base = reinterpret_cast<float4*>(T.out) + rg;
        stride = T.rows;
        add_first = T.add != 0;
      } else {
        const MPTask& t = g.mp[itm.x];
        const int64_t rg = (int64_t)itm.y * kRows + r;
        if (rg < (int64_t)t.before * t.after)
          base = reinterpret_cast<float4*>(t.out) + rg % t.before + (int64_t)t.before * t.a_out * (rg / t.before);
        stride = t.before;
        add_first = t.add != 0;
      }
      for (int u = 0; u < I.nunits; ++u, ++un) {
        const int buf = (int)(un & 1);
        const bool store = u == 0 && !add_first;
        if (!mbar_wait(&sm.bar.exready[buf], (un >> 1) & 1, kSpin) || !mbar_wait(&sm.bar.tfull, un & 1, kSpin)) {
          set_status(status, 17);
          ok = false;
          break;
        }
        fence_after_sync();
        const int er = (int)sm.ex[buf][r];
        mbar_arrive(&sm.bar.exfree[buf]);
        const int* fxg = reinterpret_cast<const int*>(tcs_image<OP>(g, itm, u, np) +
                                                      (size_t)tcs_img_steps<OP>(np) * kDig * 3 * np * 32);
        __syncwarp();
        for (int i = lane; i < 64; i += 32) fxw[i] = __ldg(fxg + i);
        __syncwarp();
        for (int n0 = c0; n0 < c1; n0 += 4) {
          // the old outputs of these four columns: their loads in flight
          // together, under the tensor-memory reads
          float4 old[4];
#pragma unroll
          for (int e = 0; e < 4; ++e)
            old[e] = (base && !store && n0 + e < I.ncols) ? base[stride * (n0 + e)] : make_float4(0.f, 0.f, 0.f, 0.f);
          __syncwarp();
          float vre[4], vim[4], lre[4], lim[4];
#pragma unroll
          for (int part = 0; part < 2; ++part) {
            float lv[kDig][4];
#pragma unroll
            for (int L = 0; L < kDig; ++L)
              if (L < NL) tmem_ld4(lane_addr + (uint32_t)(L * 2 * np + part * np + n0), lv[L]);
            tmem_wait_ld();
            float* v = part ? vim : vre;
            float* l = part ? lim : lre;
#pragma unroll
            for (int i = 0; i < 4; ++i) {
              v[i] = lv[0][i];
              l[i] = 0.f;
              if (NL > 1) df_add(v[i], l[i], lv[1][i], 0.f);
              if (NL > 2) df_add(v[i], l[i], lv[2][i], 0.f);
              float t3 = 0.f;
#pragma unroll
              for (int L = 3; L < kDig; ++L)
                if (L < NL) t3 = __fadd_rn(t3, lv[L][i]);
              l[i] = __fadd_rn(l[i], t3);
            }
          }
          if (!base) continue;
#pragma unroll
          for (int i = 0; i < 4; ++i) {
            const int col = n0 + i;
            if (col >= I.ncols) continue;
            const int fn = fxw[col];
            const int sh = (er - 126) + (fn - 126);
            float4 v;
            if (sh >= -126 && sh <= 127) {
              const float f = pow2f(sh);
              v = make_float4(vre[i] * f, lre[i] * f, vim[i] * f, lim[i] * f);
            } else {
              v = make_float4(scale2(vre[i], sh), scale2(lre[i], sh), scale2(vim[i], sh), scale2(lim[i], sh));
            }
            if (!store) {
              df_add(v.x, v.y, old[i].x, old[i].y);
              df_add(v.z, v.w, old[i].z, old[i].w);
            }
            df_norm(v.x, v.y);
            df_norm(v.z, v.w);
            if (er == 255 || fn == 255) {  // an Inf or NaN among the operands: propagate it
              const float nan = __int_as_float(0x7fffffff);
              v = make_float4(nan, nan, nan, nan);
            }
            base[stride * col] = v;
          }
        }
        fence_before_sync();
        mbar_arrive(&sm.bar.tempty);
      }
    }
  }
  fence_before_sync();
  __syncthreads();
  if (warp == 4) {
    fence_after_sync();
    tmem_dealloc(tmem, 512u);
  }
}

int g_tc_sms = 0;

cudaError_t tc_grid(int64_t n_tiles, unsigned* grid) {
  if (!g_tc_sms) {
    int dev = 0, sms = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
    g_tc_sms = sms;
  }
  *grid = (unsigned)(n_tiles < g_tc_sms ? n_tiles : g_tc_sms);
  return cudaSuccess;
}

cudaError_t launch_tf(const MPTask* tasks, const int2* tiles, int64_t first_tile, int64_t n_tiles, int* status,
                      cudaStream_t s) {
  unsigned grid = 0;
  cudaError_t e = tc_grid(n_tiles, &grid);
  if (e != cudaSuccess) return e;
  const int sm = (int)sizeof(TfSmem);
  e = cudaFuncSetAttribute(k_mp_tf, cudaFuncAttributeMaxDynamicSharedMemorySize, sm);
  if (e != cudaSuccess) return e;
  k_mp_tf<<<grid, kThreadsTc, sm, s>>>(tasks, tiles, first_tile, n_tiles, status);
  return cudaGetLastError();
}

template <int OP>
cudaError_t launch_tcs(const TcsArgs& g, const int2* img_units, int64_t first_unit, int64_t n_units, cudaStream_t s) {
  if (n_units > 0) k_tcs_img<OP><<<(unsigned)n_units, 256, 0, s>>>(g, img_units, first_unit);
  if (OP == TCS_HP) k_hp_ex<<<dim3((unsigned)g.n_items, kRows / 32), 256, 0, s>>>(g);
  unsigned grid = 0;
  cudaError_t e = tc_grid(g.n_items, &grid);
  if (e != cudaSuccess) return e;
  const int smem = (int)sizeof(TcsSmem);
  e = cudaFuncSetAttribute(k_tcs<OP>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e != cudaSuccess) return e;
  k_tcs<OP><<<grid, kThreadsTc, smem, s>>>(g);
  return cudaGetLastError();
}

}  // namespace

cudaError_t launch_hp_tc(const HPTask* tasks, const HpTcGroup* groups, const int4* items, int64_t first_item,
                         int64_t n_items, const int2* img_units, int64_t first_unit, int64_t n_units,
                         double2* ws, int* status, cudaStream_t s) {
  if (n_items <= 0) return cudaSuccess;
  TcsArgs g{};
  g.hp = tasks;
  g.groups = groups;
  g.ws = ws;
  g.items = items;
  g.item0 = first_item;
  g.n_items = n_items;
  g.status = status;
  return launch_tcs<TCS_HP>(g, img_units, first_unit, n_units, s);
}

cudaError_t launch_mp_tcs(const MPTask* tasks, const int2* tiles, int64_t first_tile, int64_t n_tiles,
                          const int* tc_tasks, int64_t first_task, int64_t n_tasks, int* status, cudaStream_t s) {
  if (n_tiles <= 0) return cudaSuccess;
  TcsArgs g{};
  g.mp = tasks;
  g.mp_tiles = tiles;
  g.mp_tasks = tc_tasks;
  g.item0 = first_tile;
  g.n_items = n_tiles;
  g.status = status;
  return launch_tcs<TCS_MP>(g, nullptr, first_task, n_tasks, s);
}

cudaError_t launch_acc_tc(const AccTask* tasks, const AccTerm* terms, const int4* items, int64_t first_item,
                          int64_t n_items, int64_t units, const int2* img_units, int64_t first_unit,
                          int64_t n_units, int* status, cudaStream_t s) {
  if (n_items <= 0) return cudaSuccess;
  TcsArgs g{};
  g.acc = tasks;
  g.terms = terms;
  g.items = items;
  g.item0 = first_item;
  g.n_items = n_items;
  g.units = units;
  g.status = status;
  return launch_tcs<TCS_ACC>(g, img_units, first_unit, n_units, s);
}

cudaError_t launch_mp_tc(bool oz, const MPTask* tasks, const int2* tiles, int64_t first_tile, int64_t n_tiles,
                         const int* tc_tasks, int64_t first_task, int64_t n_tasks, int* status, cudaStream_t s) {
  if (n_tiles <= 0) return cudaSuccess;
  if (oz) return launch_mp_tcs(tasks, tiles, first_tile, n_tiles, tc_tasks, first_task, n_tasks, status, s);
  if (n_tasks > 0) k_mp_tf_h<<<(unsigned)n_tasks, 256, 0, s>>>(tasks, tc_tasks, first_task);
  return launch_tf(tasks, tiles, first_tile, n_tiles, status, s);
}

}  // namespace qt
