// qt_umma.cu -- mode products of the mixed-precision plans on the
// fifth-generation tensor cores (tcgen05.mma, accumulators in tensor memory).
//
// out[b, j, c] = alpha sum_a h(j, a) in[b, a, c] is the GEMM Y = X H^T with
// rows r = (b, c): X is R x K (K = a_in), H^T is K x N (N = a_out), K, N <= 64.
// A CTA owns 128 consecutive rows at a time (one M = 128 accumulator tile)
// and all N columns; the complex product is four real MMAs per operand pair,
//   Y_re += X_re H_re^T - X_im H_im^T,   Y_im += X_re H_im^T + X_im H_re^T,
// the minus sign by the instruction's negate-A bit.
//
// Two arithmetics share the kernel skeleton:
//  * OZ (double-float plans, QT_PREC_DF64_TC): every operand value (hi + lo)
//    is written against the exponent of its row of X (resp. its row j of h)
//    as an integer of 49 bits cut into seven 7-bit digits q_s (s = 0 most
//    significant, |q_0| <= 128), stored in bf16 as q_s 2^(-7s), exactly.
//    Digit products are exact; pairs with s + t <= 6 are summed in fp32
//    accumulators per output, one per level L = s + t (sums of at most
//    7 * 2 * 64 * 128^2 < 2^24 in units of the level: exact) as far as
//    tensor memory holds them -- NL = min(7, 512 / (2 Np)) accumulators for
//    Np padded output columns: all seven levels for Np <= 32, five for
//    Np = 48, four for Np = 64 -- the last one taking the remaining levels
//    together.  Its fp32 rounding is the method's error: about 2^-24 of the
//    size of level NL - 1, i.e. ~1e-10 of a typical output with four
//    accumulators, ~1e-12 with five, none beyond the digits' truncation
//    (2^-44 of the row maxima) with seven.  The epilogue adds the levels in
//    double-float and scales by 2^(E_row + F_j - 14).
//  * TF (complex64 plans, QT_PREC_TF32X3): X and h (fp32) split into TF32
//    halves hi + lo; hi*hi + hi*lo + lo*hi accumulate in one fp32 sum per
//    output (split-TF32, 3 passes).
//
// Roles (288 threads): warps 0-3 produce the operand X of each 16-wide
// k-chunk into a two-stage shared-memory ring (one thread per row: first
// the row's exponent over all of K, then the digits / TF32 halves chunk by
// chunk); warp 8 allocates tensor memory, loads the h operand of the tile's
// task (prepared once per stage by a pre-pass in the exact shared-memory
// image) with bulk copies, and issues the MMAs from one thread; warps 4-7
// read the accumulators (warp 4 + q owns tensor-memory lanes 32q..32q+31,
// i.e. rows 32q..) and write the outputs.  A CTA takes a contiguous range of
// 128-row tiles, so consecutive tiles mostly share the task and its h.
// Every wait is bounded: a wait that runs out sets the status word, and the
// CTA drains its issued MMAs, frees tensor memory and returns.
#include <cuda_runtime.h>

#include <cstdint>

#include "qt_arith.cuh"
#include "qt_internal.h"
#include "qt_tc05.cuh"

namespace qt {
namespace {

using namespace tc05;

constexpr int kRows = 128;                 // rows per tile (M)
constexpr int kDig = 7;                    // digits per value (OZ)
constexpr int kThreadsTc = 288;            // 4 producer warps, 4 epilogue warps, 1 MMA warp
constexpr uint64_t kSpin = 2000000000ull;  // ns before a wait gives up (2 s)
constexpr int kChunkK = 16;                // k per ring stage

// OZ: a digit plane of one stage: 128 rows x 16 k bf16 (core layout [kc][g][8][8])
constexpr int kOzAPlane = kRows * kChunkK * 2;        // 4096 bytes
constexpr int kOzAStage = kDig * 2 * kOzAPlane;       // 57344
constexpr int kOzBMax = 4 * kDig * 2 * 64 * 32;       // 114688: K 64, N 64
// TF: a TF32 plane of one stage: 128 rows x 16 k fp32 (core layout [kc][g][8][4])
constexpr int kTfAPlane = kRows * kChunkK * 4;        // 8192 bytes
constexpr int kTfAStage = 4 * kTfAPlane;              // hi_re, hi_im, lo_re, lo_im
constexpr int kTfBMax = 4 * 4 * 64 * 64;              // 65536: K 64, N 64

template <bool OZ>
struct Cfg {
  static constexpr int AStage = OZ ? kOzAStage : kTfAStage;
  static constexpr int BMax = OZ ? kOzBMax : kTfBMax;
  static constexpr int BHeader = BMax;  // F_j (OZ) follow the digit planes in the global image
};

struct Bars {
  uint64_t full[2], empty[2], exready[2], exfree[2], tfull, tempty, bfull, drain;
  uint32_t tmem;
  int pad;
};

template <bool OZ>
struct TcSmem {
  unsigned char b[Cfg<OZ>::BMax];
  unsigned char a[2][Cfg<OZ>::AStage];
  Bars bar;
  int ex[2][kRows];    // row exponents (OZ) of the two tiles in flight
  int orow[2][kRows];  // output offset of each row (-1: past the end)
};

__device__ __forceinline__ int fexp(float v) { return (__float_as_int(v) >> 23) & 0xff; }
__device__ __forceinline__ float pow2f(int k) { return __int_as_float((k + 127) << 23); }
__device__ __forceinline__ float scale2(float v, int k) {
  if (k > 127) return (v * pow2f(127)) * pow2f(k - 127);
  if (k < -126) return (v * pow2f(-126)) * pow2f(k + 126);
  return v * pow2f(k);
}

// |hi + lo| in units of 2^(E - 49), E = eb - 126, rounded to nearest; the
// sign in neg.  eb >= 1 is the row's largest biased exponent of hi parts.
__device__ __forceinline__ uint64_t mag49(float hi, float lo, int eb, uint32_t& neg) {
  const uint32_t bh = __float_as_uint(hi), bl = __float_as_uint(lo);
  const int eh = (bh >> 23) & 0xff, el = (bl >> 23) & 0xff;
  const uint32_t mh = (bh & 0x7fffffu) | (eh ? 0x800000u : 0u);
  const uint32_t ml = (bl & 0x7fffffu) | (el ? 0x800000u : 0u);
  const int sh = max(eh, 1) - eb + 29, sl = max(el, 1) - eb + 29;
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

// digit s of a magnitude <= 2^49 as the bf16 of q_s 2^(-7s) with the sign
__device__ __forceinline__ uint16_t digit_bf16(uint64_t u, int s, uint32_t neg) {
  const uint32_t q = s == 0 ? (uint32_t)(u >> 42) : (uint32_t)(u >> (42 - 7 * s)) & 127u;
  uint32_t f = __float_as_uint(__fsub_rn(__uint_as_float(0x4B000000u | q), 8388608.0f));  // float(q), exact
  if (q) f -= (uint32_t)(7 * s) << 23;
  return (uint16_t)((f >> 16) | (neg << 15));
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
__device__ __forceinline__ int core_off(int r, int kc, int rows) { return kc * (rows / 8) * 128 + (r >> 3) * 128 + (r & 7) * 16; }

// separate level accumulators that fit tensor memory (512 columns of 2 Np each)
__device__ __forceinline__ int levels_for(int Np) { return min(kDig, 512 / (2 * Np)); }

__device__ __forceinline__ void set_status(int* status, int code) {
  if (status) atomicCAS(status, 0, code);
}

// ---------------------------------------------------------------------------
// pre-pass: the shared-memory image of h for every task of the stage
//   OZ: [ks][digit t][re/im][core layout Np x 16 k] bf16, then F_j (Np ints)
//   TF: [ks][hi_re, hi_im, lo_re, lo_im][core layout Np x 16 k] fp32
// with H^T rows j (N, padded to Np = 16 * ceil(N / 16)) and k < Kp zero-padded.
// ---------------------------------------------------------------------------
template <bool OZ>
__global__ void __launch_bounds__(256) k_mp_tc_h(const MPTask* __restrict__ tasks, const int* __restrict__ ids,
                                                 int64_t first) {
  const MPTask t = tasks[ids[first + blockIdx.x]];
  unsigned char* img = static_cast<unsigned char*>(t.oz_h);
  const float4* __restrict__ h = reinterpret_cast<const float4*>(t.h);
  const int K = t.a_in, N = t.a_out;
  const int Np = (N + 15) & ~15, Kp = (K + 15) & ~15;
  __shared__ int fx[64];
  if (OZ) {
    for (int i = threadIdx.x; i < 64; i += blockDim.x) fx[i] = 1;
    __syncthreads();
    for (int e = threadIdx.x; e < N * K; e += blockDim.x) {
      const int j = e % N, a = e / N;
      const float4 v = h[j + (int64_t)N * a];
      atomicMax(&fx[j], max(fexp(v.x), fexp(v.z)));
    }
    __syncthreads();
  }
  const int planes = OZ ? kDig * 2 : 4;
  const int esz = OZ ? 2 : 4;
  const int plane_bytes = Np * kChunkK * esz;
  // one thread per (j, k) element of H^T
  for (int e = threadIdx.x; e < Np * Kp; e += blockDim.x) {
    const int j = e % Np, k = e / Np;
    float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
    if (j < N && k < K) v = h[j + (int64_t)N * k];
    const int ks = k / kChunkK, kk = k % kChunkK;
    const int per = 16 / esz;  // elements per core row
    const int off = core_off(j, kk / per, Np) + (kk % per) * esz;
    unsigned char* base = img + (size_t)ks * planes * plane_bytes;
    if (OZ) {
      uint32_t nr = 0, ni = 0;
      const uint64_t ur = mag49(v.x, v.y, fx[j < N ? j : 0], nr);
      const uint64_t ui = mag49(v.z, v.w, fx[j < N ? j : 0], ni);
#pragma unroll
      for (int d = 0; d < kDig; ++d) {
        *reinterpret_cast<uint16_t*>(base + (size_t)(2 * d + 0) * plane_bytes + off) = digit_bf16(ur, d, nr);
        *reinterpret_cast<uint16_t*>(base + (size_t)(2 * d + 1) * plane_bytes + off) = digit_bf16(ui, d, ni);
      }
    } else {
      uint32_t hr, lr, hi_, li;
      tf32_split(v.x, hr, lr);
      tf32_split(v.z, hi_, li);
      *reinterpret_cast<uint32_t*>(base + 0 * plane_bytes + off) = hr;
      *reinterpret_cast<uint32_t*>(base + 1 * plane_bytes + off) = hi_;
      *reinterpret_cast<uint32_t*>(base + 2 * plane_bytes + off) = lr;
      *reinterpret_cast<uint32_t*>(base + 3 * plane_bytes + off) = li;
    }
  }
  if (OZ)
    for (int i = threadIdx.x; i < 64; i += blockDim.x)
      reinterpret_cast<int*>(img + Cfg<true>::BHeader)[i] = fx[i];
}

// ---------------------------------------------------------------------------
// the mode-product kernel
// ---------------------------------------------------------------------------
template <bool OZ>
__global__ void __launch_bounds__(kThreadsTc, 1) k_mp_tc(const MPTask* __restrict__ tasks,
                                                          const int2* __restrict__ tiles, int64_t tile0,
                                                          int64_t n_tiles, int* status) {
  typedef TcSmem<OZ> Sm;
  extern __shared__ __align__(128) unsigned char tc_raw[];
  Sm& sm = *reinterpret_cast<Sm*>(tc_raw);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  // contiguous tile range of this CTA
  const int64_t per = n_tiles / gridDim.x, extra = n_tiles % gridDim.x;
  const int64_t my0 = blockIdx.x * per + min((int64_t)blockIdx.x, extra);
  const int64_t my1 = my0 + per + (blockIdx.x < extra ? 1 : 0);

  if (tid == 0) {
    for (int s = 0; s < 2; ++s) {
      mbar_init(&sm.bar.full[s], 128);
      mbar_init(&sm.bar.empty[s], 1);
      mbar_init(&sm.bar.exready[s], 128);
      mbar_init(&sm.bar.exfree[s], 128);
    }
    mbar_init(&sm.bar.tfull, 1);
    mbar_init(&sm.bar.tempty, 128);
    mbar_init(&sm.bar.bfull, 1);
    mbar_init(&sm.bar.drain, 1);
    mbar_fence_init();
  }
  const uint32_t ncols = OZ ? 512u : 128u;
  if (warp == 8) tmem_alloc(&sm.bar.tmem, ncols);
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
  const uint32_t tmem = sm.bar.tmem;
  bool ok = true;

  if (warp < 4) {
    // ---------------- producers: one row each ----------------
    const int r = tid;
    uint32_t q = 0;  // chunk counter over all tiles
    for (int64_t it = my0; it < my1 && ok; ++it) {
      const int2 tl = tiles[tile0 + it];
      const MPTask t = tasks[tl.x];
      const float4* __restrict__ in = reinterpret_cast<const float4*>(t.in);
      const int K = t.a_in, N = t.a_out;
      const int64_t before = t.before, nrows = before * t.after;
      const int64_t rg = (int64_t)tl.y * kRows + r;
      const bool valid = rg < nrows;
      const int64_t b = valid ? rg % before : 0, c = valid ? rg / before : 0;
      const float4* base = in + b + before * (int64_t)K * c;
      const int buf = (int)((it - my0) & 1);
      // the epilogue of the tile two back has read ex / orow of this buffer
      if (!mbar_wait(&sm.bar.exfree[buf], (uint32_t)((((it - my0) >> 1) & 1) ^ 1), kSpin)) {
        set_status(status, 8);
        ok = false;
        break;
      }
      if (OZ) {
        int m = 1;
        if (valid)
          for (int a = 0; a < K; ++a) {
            const float4 v = __ldg(base + before * a);
            m = max(m, max(fexp(v.x), fexp(v.z)));
          }
        sm.ex[buf][r] = m;
      }
      sm.orow[buf][r] = valid ? (int)(b + before * (int64_t)N * c) : -1;
      mbar_arrive(&sm.bar.exready[buf]);
      const int eb = OZ ? sm.ex[buf][r] : 0;
      const int nks = (K + kChunkK - 1) / kChunkK;
      for (int ks = 0; ks < nks; ++ks, ++q) {
        const int s = q & 1;
        if (!mbar_wait(&sm.bar.empty[s], ((q >> 1) & 1) ^ 1, kSpin)) {
          set_status(status, 1);
          ok = false;
          break;
        }
        unsigned char* A = sm.a[s];
#pragma unroll
        for (int half = 0; half < 2; ++half) {
          float4 x[8];
#pragma unroll
          for (int i = 0; i < 8; ++i) {
            const int a = ks * kChunkK + half * 8 + i;
            x[i] = (valid && a < K) ? __ldg(base + before * a) : make_float4(0.f, 0.f, 0.f, 0.f);
          }
          if (OZ) {
            uint64_t ur[8], ui[8];
            uint32_t nr[8], ni[8];
#pragma unroll
            for (int i = 0; i < 8; ++i) {
              ur[i] = mag49(x[i].x, x[i].y, eb, nr[i]);
              ui[i] = mag49(x[i].z, x[i].w, eb, ni[i]);
            }
            const int off = core_off(r, half, kRows);
#pragma unroll
            for (int d = 0; d < kDig; ++d) {
              uint32_t wr[4], wi[4];
#pragma unroll
              for (int i = 0; i < 4; ++i) {
                wr[i] = (uint32_t)digit_bf16(ur[2 * i], d, nr[2 * i]) |
                        ((uint32_t)digit_bf16(ur[2 * i + 1], d, nr[2 * i + 1]) << 16);
                wi[i] = (uint32_t)digit_bf16(ui[2 * i], d, ni[2 * i]) |
                        ((uint32_t)digit_bf16(ui[2 * i + 1], d, ni[2 * i + 1]) << 16);
              }
              *reinterpret_cast<uint4*>(A + (2 * d + 0) * kOzAPlane + off) = make_uint4(wr[0], wr[1], wr[2], wr[3]);
              *reinterpret_cast<uint4*>(A + (2 * d + 1) * kOzAPlane + off) = make_uint4(wi[0], wi[1], wi[2], wi[3]);
            }
          } else {
            // fp32 values (complex64 storage keeps them in the hi words)
#pragma unroll
            for (int g = 0; g < 2; ++g) {  // two 16-byte core rows of 4 k each
              uint32_t hr[4], hi_[4], lr[4], li[4];
#pragma unroll
              for (int i = 0; i < 4; ++i) {
                tf32_split(x[4 * g + i].x, hr[i], lr[i]);
                tf32_split(x[4 * g + i].z, hi_[i], li[i]);
              }
              const int off = core_off(r, 2 * half + g, kRows);
              *reinterpret_cast<uint4*>(A + 0 * kTfAPlane + off) = make_uint4(hr[0], hr[1], hr[2], hr[3]);
              *reinterpret_cast<uint4*>(A + 1 * kTfAPlane + off) = make_uint4(hi_[0], hi_[1], hi_[2], hi_[3]);
              *reinterpret_cast<uint4*>(A + 2 * kTfAPlane + off) = make_uint4(lr[0], lr[1], lr[2], lr[3]);
              *reinterpret_cast<uint4*>(A + 3 * kTfAPlane + off) = make_uint4(li[0], li[1], li[2], li[3]);
            }
          }
        }
        fence_proxy_async();
        mbar_arrive(&sm.bar.full[s]);
      }
    }
  } else if (warp == 8) {
    // ---------------- MMA issue (one thread) and h loads ----------------
    if (lane == 0) {
      uint32_t q = 0, nb = 0;
      int cur = -1;
      for (int64_t it = my0; it < my1 && ok; ++it) {
        const int2 tl = tiles[tile0 + it];
        const MPTask t = tasks[tl.x];
        const int K = t.a_in, N = t.a_out;
        const int Np = (N + 15) & ~15, nks = (K + kChunkK - 1) / kChunkK;
        const int esz = OZ ? 2 : 4;
        const int planes = OZ ? kDig * 2 : 4;
        const int plane_b = Np * kChunkK * esz;  // bytes of one h plane per chunk
        const uint32_t tpar = (uint32_t)((it - my0) & 1);
        if (tl.x != cur) {
          // the previous tile's MMAs read the old h: wait until they completed
          if (it > my0 && !mbar_wait(&sm.bar.tfull, tpar ^ 1, kSpin)) {
            set_status(status, 2);
            ok = false;
            break;
          }
          const uint32_t bytes = (uint32_t)(nks * planes * plane_b);
          mbar_arrive_expect_tx(&sm.bar.bfull, bytes);
          const unsigned char* src = static_cast<const unsigned char*>(t.oz_h);
          for (uint32_t o = 0; o < bytes; o += 32768u) {
            const uint32_t n = bytes - o < 32768u ? bytes - o : 32768u;
            bulk_g2s(sm.b + o, src + o, n, &sm.bar.bfull);
          }
          if (!mbar_wait(&sm.bar.bfull, nb & 1, kSpin)) {
            set_status(status, 3);
            ok = false;
            break;
          }
          ++nb;
          cur = tl.x;
        }
        // the epilogue released the accumulators of the previous tile
        if (!mbar_wait(&sm.bar.tempty, tpar ^ 1, kSpin)) {
          set_status(status, 4);
          ok = false;
          break;
        }
        fence_after_sync();
        const uint32_t lboA = (kRows / 8) * 128, lboB = (uint32_t)(Np / 8) * 128;
        uint32_t used = 0;  // accumulators written in this tile
        for (int ks = 0; ks < nks; ++ks, ++q) {
          const int s = q & 1;
          if (!mbar_wait(&sm.bar.full[s], (q >> 1) & 1, kSpin)) {
            set_status(status, 5);
            ok = false;
            break;
          }
          fence_after_sync();
          const uint32_t a0 = smem_u32(sm.a[s]);
          const uint32_t b0 = smem_u32(sm.b) + (uint32_t)(ks * planes * plane_b);
          if (OZ) {
            const int NL = levels_for(Np);
            const uint32_t id = idesc_m128(1, Np, false), idn = idesc_m128(1, Np, true);
#pragma unroll 1
            for (int sd = 0; sd < kDig; ++sd) {
              const uint64_t are = desc_kmajor(a0 + (2 * sd + 0) * kOzAPlane, lboA, 128);
              const uint64_t aim = desc_kmajor(a0 + (2 * sd + 1) * kOzAPlane, lboA, 128);
              for (int td = 0; td + sd < kDig; ++td) {
                const int L = sd + td < NL - 1 ? sd + td : NL - 1;
                const uint64_t bre = desc_kmajor(b0 + (2 * td + 0) * plane_b, lboB, 128);
                const uint64_t bim = desc_kmajor(b0 + (2 * td + 1) * plane_b, lboB, 128);
                const uint32_t dre = tmem + (uint32_t)(L * 2 * Np), dim_ = dre + (uint32_t)Np;
                const uint32_t fre = (used >> (2 * L)) & 1, fim = (used >> (2 * L + 1)) & 1;
                mma_bf16(dre, are, bre, id, fre);
                mma_bf16(dre, aim, bim, idn, 1);
                mma_bf16(dim_, are, bim, id, fim);
                mma_bf16(dim_, aim, bre, id, 1);
                used |= 3u << (2 * L);
              }
            }
          } else {
            const uint32_t id = idesc_m128(2, Np, false), idn = idesc_m128(2, Np, true);
            const uint32_t lboA4 = (kRows / 8) * 128;  // kc stride of a 16-k fp32 plane: [kc (4)][g][8][4]
#pragma unroll 1
            for (int h8 = 0; h8 < 2; ++h8) {  // two MMAs of k = 8 per chunk
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
              const uint32_t f = used;  // 0 only for the first MMAs of the tile
              // lo x hi and hi x lo first, then hi x hi
              mma_tf32(dre, alr, bhr, id, f);
              mma_tf32(dre, ali, bhi, idn, 1);
              mma_tf32(dim_, alr, bhi, id, f);
              mma_tf32(dim_, ali, bhr, id, 1);
              mma_tf32(dre, ahr, blr, id, 1);
              mma_tf32(dre, ahi, bli, idn, 1);
              mma_tf32(dim_, ahr, bli, id, 1);
              mma_tf32(dim_, ahi, blr, id, 1);
              mma_tf32(dre, ahr, bhr, id, 1);
              mma_tf32(dre, ahi, bhi, idn, 1);
              mma_tf32(dim_, ahr, bhi, id, 1);
              mma_tf32(dim_, ahi, bhr, id, 1);
              used = 1;
            }
          }
          commit(&sm.bar.empty[s]);  // the stage is free once these MMAs completed
        }
        if (!ok) break;
        commit(&sm.bar.tfull);
      }
      // drain: every MMA issued by this thread completed before tensor memory is freed
      commit(&sm.bar.drain);
      if (!mbar_wait(&sm.bar.drain, 0, kSpin)) set_status(status, 6);
    }
  } else {
    // ---------------- epilogue: warp 4 + qd reads lanes 32 qd .. ----------------
    const int qd = warp - 4;
    const int r = 32 * qd + lane;
    const uint32_t lane_addr = tmem + ((uint32_t)(32 * qd) << 16);
    for (int64_t it = my0; it < my1 && ok; ++it) {
      const int2 tl = tiles[tile0 + it];
      const MPTask t = tasks[tl.x];
      const int N = t.a_out, Np = (N + 15) & ~15;
      const int64_t before = t.before;
      const int buf = (int)((it - my0) & 1);
      const uint32_t tpar = (uint32_t)((it - my0) & 1);
      if (!mbar_wait(&sm.bar.exready[buf], (uint32_t)(((it - my0) >> 1) & 1), kSpin) ||
          !mbar_wait(&sm.bar.tfull, tpar, kSpin)) {
        set_status(status, 7);
        ok = false;
        break;
      }
      fence_after_sync();
      const int ro = sm.orow[buf][r];
      const int er = OZ ? sm.ex[buf][r] : 0;
      mbar_arrive(&sm.bar.exfree[buf]);
      const bool live = ro >= 0;
      const int* fxg = OZ ? reinterpret_cast<const int*>(static_cast<const unsigned char*>(t.oz_h) + Cfg<true>::BHeader)
                          : nullptr;
      float4* out = reinterpret_cast<float4*>(t.out);
      const bool unit = t.alpha.x == 1.0 && t.alpha.y == 0.0;
      for (int j0 = 0; j0 < Np; j0 += 8) {
        __syncwarp();  // the tensor-memory loads below are warp-collective
        float vre[8], vim[8], lre[8], lim[8];
        if (OZ) {
          const int NL = levels_for(Np);
          tmem_ld8(lane_addr + (uint32_t)j0, vre);
          tmem_ld8(lane_addr + (uint32_t)(Np + j0), vim);
          tmem_wait_ld();
#pragma unroll
          for (int i = 0; i < 8; ++i) lre[i] = lim[i] = 0.f;
          for (int L = 1; L < NL; ++L) {  // warp-uniform
            float ar[8], ai[8];
            tmem_ld8(lane_addr + (uint32_t)(L * 2 * Np + j0), ar);
            tmem_ld8(lane_addr + (uint32_t)(L * 2 * Np + Np + j0), ai);
            tmem_wait_ld();
#pragma unroll
            for (int i = 0; i < 8; ++i) {
              df_add(vre[i], lre[i], ar[i], 0.f);
              df_add(vim[i], lim[i], ai[i], 0.f);
            }
          }
        } else {
          tmem_ld8(lane_addr + (uint32_t)j0, vre);
          tmem_ld8(lane_addr + (uint32_t)(Np + j0), vim);
          tmem_wait_ld();
#pragma unroll
          for (int i = 0; i < 8; ++i) lre[i] = lim[i] = 0.f;
        }
#pragma unroll
        for (int i = 0; i < 8; ++i) {
          const int j = j0 + i;
          if (!live || j >= N) continue;
          float4 v;
          if (OZ) {
            const int fj = __ldg(fxg + j);
            const int sh = (er - 126) + (fj - 126) - 14;
            v = make_float4(scale2(vre[i], sh), scale2(lre[i], sh), scale2(vim[i], sh), scale2(lim[i], sh));
            df_norm(v.x, v.y);
            df_norm(v.z, v.w);
            if (!unit) v = DF64::mul(DF64::coef(t.alpha), v);
            if (er == 255 || fj == 255) {  // an Inf or NaN in the row: propagate it
              const float nan = __int_as_float(0x7fffffff);
              v = make_float4(nan, nan, nan, nan);
            }
          } else {
            v = make_float4(vre[i], 0.f, vim[i], 0.f);
            if (!unit) v = C32::mul(C32::coef(t.alpha), v);
          }
          out[ro + before * j] = v;
        }
      }
      fence_before_sync();
      mbar_arrive(&sm.bar.tempty);
    }
  }
  fence_before_sync();
  __syncthreads();
  if (warp == 8) {
    fence_after_sync();
    tmem_dealloc(tmem, ncols);
  }
}

int g_tc_sms = 0;

}  // namespace

cudaError_t launch_mp_tc(bool oz, const MPTask* tasks, const int2* tiles, int64_t first_tile, int64_t n_tiles,
                         const int* tc_tasks, int64_t first_task, int64_t n_tasks, int* status, cudaStream_t s) {
  if (n_tiles <= 0) return cudaSuccess;
  if (!g_tc_sms) {
    int dev = 0, sms = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
    g_tc_sms = sms;
  }
  const unsigned grid = (unsigned)(n_tiles < g_tc_sms ? n_tiles : g_tc_sms);
  if (oz) {
    if (n_tasks > 0) k_mp_tc_h<true><<<(unsigned)n_tasks, 256, 0, s>>>(tasks, tc_tasks, first_task);
    const int sm = (int)sizeof(TcSmem<true>);
    cudaError_t e = cudaFuncSetAttribute(k_mp_tc<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm);
    if (e != cudaSuccess) return e;
    k_mp_tc<true><<<grid, kThreadsTc, sm, s>>>(tasks, tiles, first_tile, n_tiles, status);
  } else {
    if (n_tasks > 0) k_mp_tc_h<false><<<(unsigned)n_tasks, 256, 0, s>>>(tasks, tc_tasks, first_task);
    const int sm = (int)sizeof(TcSmem<false>);
    cudaError_t e = cudaFuncSetAttribute(k_mp_tc<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm);
    if (e != cudaSuccess) return e;
    k_mp_tc<false><<<grid, kThreadsTc, sm, s>>>(tasks, tiles, first_tile, n_tiles, status);
  }
  return cudaGetLastError();
}

}  // namespace qt
