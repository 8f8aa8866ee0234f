// qt_kernels.cu -- complex128 kernels of the H.Psi sweep for sm_103a.
//
// GB300 executes FP64 at ~1.2 TFLOP/s (1/61 of its FP32 rate), so every
// complex128 contraction here is bound by the FP64 pipe, not by HBM: a
// complex multiply-add needs 4 DFMA but at most 32 bytes of operands, which
// L1/L2 deliver far faster than the DFMA units consume them.  The kernels are
// therefore plain SIMT loops with coalesced 16-byte complex loads, shared
// memory staging where an operand is reused by a whole tile, several
// independent accumulators per thread for instruction-level parallelism, and
// fixed summation orders (no atomics: results are bit-identical run to run).
//
// Batched launches: each kernel reads a task table and a tile table; block b
// processes tile b.  The planner (qt_plan.cpp) builds both once per tree.
#include <algorithm>
#include <cmath>
#include <mutex>
#include <type_traits>

#include <cuda.h>

#include "qt_arith.cuh"
#include "qt_internal.h"

namespace qt {
namespace {

constexpr int kThreads = 256;
constexpr int kMpTile = kThreads;  // slots (up to four outputs each) per mode-product tile, as in the planner
constexpr int kHpMaxDim = 112;  // largest bond the planner admits
constexpr int kHpK = 16;
constexpr int kAccRows = 64;
constexpr int kCvtPerThread = 8;  // 2048 elements per tile, as in the planner

__device__ __forceinline__ double2 cz() { return cz64(); }
__device__ __forceinline__ double2 cmul(double2 a, double2 b) { return cmul64(a, b); }
__device__ __forceinline__ void cfma(double2& acc, double2 a, double2 b) { cfma64(acc, a, b); }
__device__ __forceinline__ void cfmac(double2& acc, double2 a, double2 b) { cfmac64(acc, a, b); }
__device__ __forceinline__ double2 cadd(double2 a, double2 b) { return cadd64(a, b); }

// ---------------------------------------------------------------------------
// Mode-k product (matvec / matrixTensor): one thread per slot (b, j0..j0+3, c)
// of up to four outputs that share the input fiber in[b, :, c]: per a one
// input load and four h loads feed four products.  Slots run b fastest:
// along higher modes consecutive threads read consecutive input elements
// (coalesced) and share h; along mode 0 (before = 1) they read consecutive
// groups of h's rows and share the input fiber.
// ---------------------------------------------------------------------------
template <class P>
__device__ __forceinline__ void mp_tile(const MPTask& t, int64_t slot0) {
  typedef typename P::S S;
  typedef typename P::A A;
  const S* __restrict__ in = reinterpret_cast<const S*>(t.in);
  const S* __restrict__ h = reinterpret_cast<const S*>(t.h);
  S* out = reinterpret_cast<S*>(t.out);
  const int nq = (t.a_out + 3) / 4;
  const int64_t before = t.before;
  const int64_t slot = slot0 + threadIdx.x;
  if (slot >= before * nq * t.after) return;
  const int64_t b = slot % before;
  const int64_t r = slot / before;
  const int j0 = 4 * (int)(r % nq);
  const int64_t c = r / nq;
  const int nj = t.a_out - j0 < 4 ? t.a_out - j0 : 4;
  const S* ip = in + b + before * t.a_in * c;  // in[b, a, c] = ip[before a]
  const bool unit = t.alpha.x == 1.0 && t.alpha.y == 0.0;
  const typename P::C alpha = P::coef(t.alpha);
  S res[4];
  if (t.diag) {
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int j = j0 + (q < nj ? q : 0);
      res[q] = P::mul(P::ld(h + j), P::ld(ip + before * j));
    }
  } else {
    A acc[4] = {P::zero(), P::zero(), P::zero(), P::zero()};
    const S* hp = h + j0;  // h(j, a) = h[j + a_out a]
    const int64_t hs = t.a_out;
    for (int a = 0; a < t.a_in; ++a) {
      const S x = P::ld(ip);
      S h0[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) h0[q] = P::ld(hp + (q < nj ? q : 0));
      ip += before;
      hp += hs;
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        P::mac(acc[q], h0[q], x);
        if (a & 1) P::norm(acc[q]);
      }
    }
#pragma unroll
    for (int q = 0; q < 4; ++q) res[q] = P::fin(acc[q]);
  }
#pragma unroll
  for (int q = 0; q < 4; ++q)
    if (q < nj) {
      const int64_t o = b + before * ((j0 + q) + (int64_t)t.a_out * c);
      const S v = unit ? res[q] : P::scale(alpha, res[q]);
      out[o] = t.add ? P::plus(out[o], v) : v;
    }
}

template <class P>
__global__ void __launch_bounds__(kThreads) k_mp(const MPTask* __restrict__ tasks,
                                                 const int2* __restrict__ tiles, int64_t tile0) {
  const int2 tl = tiles[tile0 + blockIdx.x];
  const MPTask t = tasks[tl.x];
  mp_tile<P>(t, tl.y);
}

__global__ void __launch_bounds__(kThreads) k_mp_single(MPTask t) {
  mp_tile<F64>(t, (int64_t)blockIdx.x * kMpTile);
}

// ---------------------------------------------------------------------------
// Hole product (rhomat / contraction): S(i, j) = sum_k conj(A[k; i]) B[k; j]
// with k = (b, c).  A 32 x 32 output tile per block, 2 x 2 outputs per
// thread; A and B are staged through shared memory 16 k-rows at a time with
// coalesced loads (along b when before > 1, along i when before == 1).
// ---------------------------------------------------------------------------
template <class P>
__device__ __forceinline__ void hp_tile(const HPTask& t, int mt0) {
  // Output S is split into 2 x 2 micro-tiles {i, i + mi} x {j, j + mj}
  // (mi = ceil(aA/2), mj = ceil(aB/2)), numbered column-major over the
  // mi x mj grid; thread x of the block owns micro-tile mt0 + x.  Adjacent
  // threads read adjacent rows of the staged operands (conflict-free shared
  // loads).  Threads past the last micro-tile form whole idle warps (they
  // only help stage operands), so no lanes idle inside a warp.
  typedef typename P::S S;
  typedef typename P::A A;
  extern __shared__ __align__(16) unsigned char hp_smem[];
  const S* __restrict__ Ap = reinterpret_cast<const S*>(t.A);
  const S* __restrict__ Bp = reinterpret_cast<const S*>(t.B);
  S* Sp = reinterpret_cast<S*>(t.S);
  const int before = t.before;
  const int aA = t.a, aB = t.aB > 0 ? t.aB : t.a;
  S* sA = reinterpret_cast<S*>(hp_smem);   // [kHpK][aA]
  S* sB = sA + kHpK * aA;                  // [kHpK][aB]
  const int64_t K = (int64_t)before * t.after;
  const int64_t sliceA = (int64_t)before * aA, sliceB = (int64_t)before * aB;
  const int mi = (aA + 1) / 2, mj = (aB + 1) / 2;
  const int mt = mt0 + threadIdx.x;
  const bool active = mt < mi * mj;
  const int i = active ? mt % mi : 0;
  const int j = active ? mt / mi : 0;
  const bool has_i1 = i + mi < aA, has_j1 = j + mj < aB;
  const int i1 = has_i1 ? i + mi : i, j1 = has_j1 ? j + mj : j;
  A acc00 = P::zero(), acc01 = P::zero(), acc10 = P::zero(), acc11 = P::zero();
  const int nA = kHpK * aA, nAB = kHpK * (aA + aB);
  for (int64_t k0 = 0; k0 < K; k0 += kHpK) {
    for (int e = threadIdx.x; e < nAB; e += kThreads) {
      const bool isA = e < nA;
      const int ee = isA ? e : e - nA;
      const int ncol = isA ? aA : aB;
      int kk, ii;
      if (before == 1) {
        ii = ee % ncol;
        kk = ee / ncol;
      } else {
        kk = ee % kHpK;
        ii = ee / kHpK;
      }
      const int64_t k = k0 + kk;
      S v = P::zero();
      if (k < K) {
        const int64_t b = k % before, c = k / before;
        v = isA ? P::ld(Ap + b + (int64_t)before * ii + sliceA * c)
                : P::ld(Bp + b + (int64_t)before * ii + sliceB * c);
      }
      (isA ? sA : sB)[kk * ncol + ii] = v;
    }
    __syncthreads();
    if (active) {
#pragma unroll 4
      for (int kk = 0; kk < kHpK; ++kk) {
        const S a0 = sA[kk * aA + i], a1 = sA[kk * aA + i1];
        const S b0 = sB[kk * aB + j], b1 = sB[kk * aB + j1];
        P::macc(acc00, a0, b0);
        P::macc(acc10, a1, b0);
        P::macc(acc01, a0, b1);
        P::macc(acc11, a1, b1);
        if (kk & 1) {
          P::norm(acc00);
          P::norm(acc10);
          P::norm(acc01);
          P::norm(acc11);
        }
      }
    }
    __syncthreads();
  }
  if (!active) return;
  Sp[i + (int64_t)aA * j] = P::fin(acc00);
  if (has_i1) Sp[i1 + (int64_t)aA * j] = P::fin(acc10);
  if (has_j1) Sp[i + (int64_t)aA * j1] = P::fin(acc01);
  if (has_i1 && has_j1) Sp[i1 + (int64_t)aA * j1] = P::fin(acc11);
}

__global__ void __launch_bounds__(kThreads) k_hp_single(HPTask t) {
  hp_tile<F64>(t, blockIdx.x * kThreads);
}

inline int hp_smem_bytes(int aA, int aB) { return kHpK * (aA + aB) * 16; }

// ---------------------------------------------------------------------------
// Hole products of the sweep, split over the reduction index k.  A block owns
// one output tile of up to 64 x 64 and one range of kchunk rows of k; its
// thread (tx, ty) of the TA x TB grid owns the R x C outputs
// {tx + TA r} x {ty + TB c} (R, C in 1..4 chosen per task by the planner so
// that small tiles still occupy most of the 256 threads; one kernel per
// shape, launched once per shape present in a stage).  The operand rows
// move into shared memory 16 at a time with cp.async into two buffers: the
// next rows load while the current ones are consumed, one barrier per 16
// rows.  A task cut into several k ranges writes normalised partial tiles to
// the workspace; k_hp_sum adds them in range order (deterministic).
// ---------------------------------------------------------------------------
constexpr int kHpTile = 64;
constexpr int kHpRows = 16;
constexpr int kHpSmem = 2 * 2 * kHpRows * kHpTile * 16;  // two buffers of A and B rows: 64 KiB

__device__ __forceinline__ void cp_async16(void* smem, const void* gmem, bool valid) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
  const int n = valid ? 16 : 0;  // 0: fill the 16 bytes with zeros, read nothing
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(sa), "l"(gmem), "r"(n) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

// one block: output tile tl.y, reduction range tl.z of task t
template <class P, int R, int C>
__device__ __forceinline__ void hp_split_tile(const HPTask& t, const int4 tl, typename P::S* __restrict__ ws) {
  typedef typename P::S S;
  typedef typename P::A A;
  extern __shared__ __align__(16) unsigned char hp_smem[];
  S* sm = reinterpret_cast<S*>(hp_smem);  // [buffer][A rows | B rows][kHpRows][kHpTile]
  const int aA = t.a, aB = t.aB > 0 ? t.aB : t.a;
  const int nti = (aA + kHpTile - 1) / kHpTile;
  const int ti0 = (tl.y % nti) * kHpTile, tj0 = (tl.y / nti) * kHpTile;
  const int mA = min(kHpTile, aA - ti0), mB = min(kHpTile, aB - tj0);
  const int TA = (mA + R - 1) / R, TB = (mB + C - 1) / C;
  const int before = t.before;
  const int64_t K = (int64_t)before * t.after;
  const int64_t kb = (int64_t)tl.z * t.kchunk;
  const int64_t ke = min(K, kb + (int64_t)t.kchunk);
  const S* __restrict__ Ap = reinterpret_cast<const S*>(t.A);
  const S* __restrict__ Bp = reinterpret_cast<const S*>(t.B);
  const int64_t sliceA = (int64_t)before * aA, sliceB = (int64_t)before * aB;
  const int tid = threadIdx.x;
  const bool active = tid < TA * TB;
  const int tx = active ? tid % TA : 0, ty = active ? tid / TA : 0;
  const int wA = R * TA, wB = C * TB;  // staged columns (zero beyond the tile; <= 64)
  const int nA = kHpRows * wA, nAB = kHpRows * (wA + wB);
  auto stage = [&](int buf, int64_t k0) {
    S* dA = sm + buf * 2 * kHpRows * kHpTile;
    S* dB = dA + kHpRows * kHpTile;
    for (int e = tid; e < nAB; e += kThreads) {
      const bool isA = e < nA;
      const int ee = isA ? e : e - nA;
      const int w = isA ? wA : wB;
      int kk, ii;
      if (before == 1) {  // consecutive columns are contiguous
        ii = ee % w;
        kk = ee / w;
      } else {  // consecutive rows are contiguous
        kk = ee % kHpRows;
        ii = ee / kHpRows;
      }
      const int64_t k = k0 + kk;
      const bool ok = k < ke && ii < (isA ? mA : mB);
      const S* src = isA ? Ap : Bp;
      if (ok) {
        const int64_t b = k % before, c = k / before;
        src += b + (int64_t)before * ((isA ? ti0 : tj0) + ii) + (isA ? sliceA : sliceB) * c;
      }
      cp_async16((isA ? dA : dB) + kk * kHpTile + ii, src, ok);
    }
    cp_async_commit();
  };
  A acc[R][C];
#pragma unroll
  for (int r = 0; r < R; ++r)
#pragma unroll
    for (int c = 0; c < C; ++c) acc[r][c] = P::zero();
  const int64_t nchunks = (ke - kb + kHpRows - 1) / kHpRows;
  if (nchunks > 0) stage(0, kb);
  for (int64_t ch = 0; ch < nchunks; ++ch) {
    cp_async_wait<0>();
    // chunk ch has landed, and every thread is done with buffer (ch + 1) & 1
    __syncthreads();
    if (ch + 1 < nchunks) stage((int)((ch + 1) & 1), kb + (ch + 1) * kHpRows);
    if (active) {
      const S* cA = sm + (ch & 1) * 2 * kHpRows * kHpTile;
      const S* cB = cA + kHpRows * kHpTile;
#pragma unroll 2
      for (int kk = 0; kk < kHpRows; ++kk) {
        S a[R], b[C];
#pragma unroll
        for (int r = 0; r < R; ++r) a[r] = cA[kk * kHpTile + tx + TA * r];
#pragma unroll
        for (int c = 0; c < C; ++c) b[c] = cB[kk * kHpTile + ty + TB * c];
#pragma unroll
        for (int r = 0; r < R; ++r)
#pragma unroll
          for (int c = 0; c < C; ++c) P::macc(acc[r][c], a[r], b[c]);
        if (kk & 1) {
#pragma unroll
          for (int r = 0; r < R; ++r)
#pragma unroll
            for (int c = 0; c < C; ++c) P::norm(acc[r][c]);
        }
      }
    }
  }
  if (!active) return;
  S* Sp = reinterpret_cast<S*>(t.S);
  const int64_t nS = (int64_t)aA * aB;
#pragma unroll
  for (int r = 0; r < R; ++r)
#pragma unroll
    for (int c = 0; c < C; ++c) {
      const int i = tx + TA * r, j = ty + TB * c;
      if (i < mA && j < mB) {
        const int64_t o = (ti0 + i) + (int64_t)aA * (tj0 + j);
        if (t.splits <= 1)
          Sp[o] = P::fin(acc[r][c]);
        else
          ws[t.ws + (int64_t)tl.z * nS + o] = P::fin(acc[r][c]);
      }
    }
}

template <class P, int R, int C>
__global__ void __launch_bounds__(kThreads, R * C > 9 ? 2 : 3)
    k_hp(const HPTask* __restrict__ tasks, const int4* __restrict__ tiles, int64_t tile0,
         typename P::S* __restrict__ ws) {
  const int4 tl = tiles[tile0 + blockIdx.x];
  const HPTask t = tasks[tl.x];
  hp_split_tile<P, R, C>(t, tl, ws);
}

// one task passed by value: block b covers output tile b % ntiles, range b / ntiles
template <class P, int R, int C>
__global__ void __launch_bounds__(kThreads, R * C > 9 ? 2 : 3)
    k_hp_one(HPTask t, int ntiles, typename P::S* __restrict__ ws) {
  hp_split_tile<P, R, C>(t, make_int4(0, (int)(blockIdx.x % ntiles), (int)(blockIdx.x / ntiles), 0), ws);
}

template <class P>
__global__ void __launch_bounds__(kThreads) k_hp_sum_one(HPTask t, const typename P::S* __restrict__ ws) {
  typedef typename P::S S;
  typedef typename P::A A;
  const int aB = t.aB > 0 ? t.aB : t.a;
  const int64_t n = (int64_t)t.a * aB;
  S* Sp = reinterpret_cast<S*>(t.S);
  for (int64_t e = (int64_t)blockIdx.x * kThreads + threadIdx.x; e < n; e += (int64_t)gridDim.x * kThreads) {
    A acc = P::zero();
    for (int z = 0; z < t.splits; ++z) P::add(acc, ws[t.ws + z * n + e]);
    Sp[e] = P::fin(acc);
  }
}

// S = sum over the k ranges of the partial tiles, in range order; kHpSumChunks
// blocks of 256 outputs per task (the loads of four ranges in flight)
constexpr int kHpSumChunks = 16;
template <class P>
__global__ void __launch_bounds__(kThreads) k_hp_sum(const HPTask* __restrict__ tasks, int64_t task0,
                                                     const typename P::S* __restrict__ ws) {
  typedef typename P::S S;
  typedef typename P::A A;
  const HPTask t = tasks[task0 + blockIdx.x / kHpSumChunks];
  if (t.splits <= 1) return;
  const int aB = t.aB > 0 ? t.aB : t.a;
  const int64_t n = (int64_t)t.a * aB;
  S* Sp = reinterpret_cast<S*>(t.S);
  for (int64_t e = (int64_t)(blockIdx.x % kHpSumChunks) * kThreads + threadIdx.x; e < n;
       e += (int64_t)kHpSumChunks * kThreads) {
    A acc = P::zero();
#pragma unroll 4
    for (int z = 0; z < t.splits; ++z) P::add(acc, ws[t.ws + z * n + e]);
    Sp[e] = P::fin(acc);
  }
}

// ---------------------------------------------------------------------------
// Last-mode accumulation (multStateAB summed over terms):
//   out[r, j] (+)= alpha * sum_t sum_j' H_t(j, j') X_t[r, j'].
// 64 rows x 16 columns per block; a warp covers 32 consecutive rows (coalesced
// X loads) of 4 columns (H loads broadcast across the warp).
// ---------------------------------------------------------------------------
template <class P>
__global__ void __launch_bounds__(kThreads) k_acc(const AccTask* __restrict__ tasks,
                                                  const AccTerm* __restrict__ terms,
                                                  const int4* __restrict__ tiles, int64_t tile0) {
  typedef typename P::S S;
  typedef typename P::A A;
  const int4 tl = tiles[tile0 + blockIdx.x];
  const AccTask t = tasks[tl.x];
  const int r = tl.y + threadIdx.x % kAccRows;
  const int jb = tl.z + (threadIdx.x / kAccRows) * 4;
  const bool rv = r < t.rows;
  const int d = t.d;
  if (jb >= d) return;  // the whole warp lies past the last column
  const int nq = d - jb < 4 ? d - jb : 4;  // uniform across the warp
  const int64_t rows = t.rows;
  A acc[4] = {P::zero(), P::zero(), P::zero(), P::zero()};
  for (int s = 0; s < t.count; ++s) {
    const AccTerm T = terms[t.first + s];
    const S* X = reinterpret_cast<const S*>(T.X);
    if (T.H == nullptr) {
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int j = jb + q;
        if (rv && j < d) P::add(acc[q], P::ld(X + r + rows * j));
      }
    } else {
      const S* H = reinterpret_cast<const S*>(T.H);
      const S* hrow[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) hrow[q] = H + (jb + q < d ? jb + q : 0);
      if (nq == 4) {
        for (int jp = 0; jp < d; ++jp) {
          const S x = rv ? P::ld(X + r + rows * jp) : P::zero();
#pragma unroll
          for (int q = 0; q < 4; ++q) P::mac(acc[q], P::ld(hrow[q] + (int64_t)d * jp), x);
          if (jp & 1) {
#pragma unroll
            for (int q = 0; q < 4; ++q) P::norm(acc[q]);
          }
        }
      } else {
        for (int jp = 0; jp < d; ++jp) {
          const S x = rv ? P::ld(X + r + rows * jp) : P::zero();
#pragma unroll
          for (int q = 0; q < 4; ++q)
            if (q < nq) P::mac(acc[q], P::ld(hrow[q] + (int64_t)d * jp), x);
          if (jp & 1) {
#pragma unroll
            for (int q = 0; q < 4; ++q) P::norm(acc[q]);
          }
        }
      }
    }
  }
  const double2 alpha64 = t.alpha_ptr ? *t.alpha_ptr : t.alpha;
  const typename P::C alpha = P::coef(alpha64);
  S* out = reinterpret_cast<S*>(t.out);
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int j = jb + q;
    if (rv && j < d) {
      const S v = P::scale(alpha, P::fin(acc[q]));
      S* p = out + r + rows * j;
      *p = t.add ? P::plus(*p, v) : v;
    }
  }
}

// out = sum_t c_t M_t (d x d), one block per output matrix.
template <class P>
__global__ void __launch_bounds__(kThreads) k_lin(const LinTask* __restrict__ tasks,
                                                  const LinTerm* __restrict__ terms, int64_t task0) {
  typedef typename P::S S;
  const LinTask t = tasks[task0 + blockIdx.x];
  const int dd = t.d * t.d;
  S* out = reinterpret_cast<S*>(t.out);
  for (int e = threadIdx.x; e < dd; e += kThreads) {
    typename P::A acc = P::zero();
    for (int s = 0; s < t.count; ++s) {
      const LinTerm T = terms[t.first + s];
      P::cmac(acc, P::coef(T.c), P::ld(reinterpret_cast<const S*>(T.M) + e));
      P::norm(acc);
    }
    out[e] = P::fin(acc);
  }
}

// out(i, j) = sum_t sum_k A_t(i, k) op(B_t)(k, j), one output element per
// thread, 256 per block (tiles of the task list).
template <class P>
__global__ void __launch_bounds__(kThreads) k_mm(const MMTask* __restrict__ tasks, const MMTerm* __restrict__ terms,
                                                 const int2* __restrict__ tiles, int64_t tile0) {
  typedef typename P::S S;
  const int2 tl = tiles[tile0 + blockIdx.x];
  const MMTask t = tasks[tl.x];
  const int d = t.d;
  const int e = tl.y + threadIdx.x;
  if (e >= d * d) return;
  const int i = e % d, j = e / d;
  // four independent accumulators over k mod 4 (instruction-level parallelism)
  typename P::A acc[4] = {P::zero(), P::zero(), P::zero(), P::zero()};
  const int64_t bs = t.trans_b ? d : 1;  // B element (k, j): B[j + d k] or B[k + d j]
  for (int s = 0; s < t.count; ++s) {
    const MMTerm T = terms[t.first + s];
    const S* A = reinterpret_cast<const S*>(T.A) + i;
    const S* B = reinterpret_cast<const S*>(T.B) + (t.trans_b ? j : (int64_t)d * j);
    int k = 0;
    for (; k + 3 < d; k += 4) {
      S a[4], b[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        a[q] = P::ld(A + (int64_t)d * (k + q));
        b[q] = P::ld(B + bs * (k + q));
      }
#pragma unroll
      for (int q = 0; q < 4; ++q) P::mac(acc[q], a[q], b[q]);
      if (k & 4) {
#pragma unroll
        for (int q = 0; q < 4; ++q) P::norm(acc[q]);
      }
    }
    for (; k < d; ++k) P::mac(acc[0], P::ld(A + (int64_t)d * k), P::ld(B + bs * k));
#pragma unroll
    for (int q = 0; q < 4; ++q) P::norm(acc[q]);
  }
#pragma unroll
  for (int q = 1; q < 4; ++q) P::add(acc[0], P::fin(acc[q]));
  reinterpret_cast<S*>(t.out)[e] = P::fin(acc[0]);
}

// Energy-gradient preparation: M3 = Eout - E rho per node, alpha = 1/S00.
template <class P>
__global__ void __launch_bounds__(kThreads) k_grad(const GradTask* __restrict__ tasks, int64_t task0) {
  typedef typename P::S S;
  const GradTask t = tasks[task0 + blockIdx.x];
  const double E = t.h00->x / t.s00->x;
  const typename P::C mE = P::coef(make_double2(-E, 0.0));
  const S* eout = reinterpret_cast<const S*>(t.eout);
  const S* rho = reinterpret_cast<const S*>(t.rho);
  S* m3 = reinterpret_cast<S*>(t.m3);
  for (int e = threadIdx.x; e < t.d * t.d; e += kThreads) {
    typename P::A acc = eout ? P::ld(eout + e) : P::zero();
    P::cmac(acc, mE, P::ld(rho + e));
    m3[e] = P::fin(acc);
  }
  if (t.write_alpha && threadIdx.x == 0) *t.alpha = make_double2(1.0 / t.s00->x, 0.0);
}

// Precision conversions: dir 0 complex128 -> double-float, dir 1 back.
__global__ void __launch_bounds__(kThreads) k_cvt(const CvtTask* __restrict__ tasks,
                                                  const int2* __restrict__ tiles, int64_t tile0) {
  const int2 tl = tiles[tile0 + blockIdx.x];
  const CvtTask t = tasks[tl.x];
  // all loads of the thread first (eight 16-byte loads in flight), then convert
  if (t.dir == 0) {
    double2 v[kCvtPerThread];
#pragma unroll
    for (int q = 0; q < kCvtPerThread; ++q) {
      const int64_t i = tl.y + threadIdx.x + (int64_t)q * kThreads;
      v[q] = i < t.n ? __ldg(reinterpret_cast<const double2*>(t.src) + i) : make_double2(0.0, 0.0);
    }
#pragma unroll
    for (int q = 0; q < kCvtPerThread; ++q) {
      const int64_t i = tl.y + threadIdx.x + (int64_t)q * kThreads;
      if (i < t.n) {
        const float2 r = df_split(v[q].x), m = df_split(v[q].y);
        reinterpret_cast<float4*>(t.dst)[i] = make_float4(r.x, r.y, m.x, m.y);
      }
    }
  } else {
    float4 w[kCvtPerThread];
#pragma unroll
    for (int q = 0; q < kCvtPerThread; ++q) {
      const int64_t i = tl.y + threadIdx.x + (int64_t)q * kThreads;
      w[q] = i < t.n ? __ldg(reinterpret_cast<const float4*>(t.src) + i) : make_float4(0.f, 0.f, 0.f, 0.f);
    }
#pragma unroll
    for (int q = 0; q < kCvtPerThread; ++q) {
      const int64_t i = tl.y + threadIdx.x + (int64_t)q * kThreads;
      if (i < t.n)
        reinterpret_cast<double2*>(t.dst)[i] =
            make_double2((double)w[q].x + (double)w[q].y, (double)w[q].z + (double)w[q].w);
    }
  }
}

// ---------------------------------------------------------------------------
// Regularised inverse of a Hermitian matrix (SpectralDecompositionTree::
// calculate + invert): parallel cyclic Jacobi with a round-robin pairing
// (every round rotates d/2 disjoint index pairs at once), then
//   rhoinv = U diag(1 / (w + eps*exp(-w/eps))) U^dagger.
// One block per matrix; A lives in shared memory, U in global scratch.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void rr_pair(int m, int r, int i, int& p, int& q) {
  // circle method over m (even) indices, round r in [0, m-1), pair i in [0, m/2)
  if (i == 0) {
    p = r;
    q = m - 1;
  } else {
    p = (r + i) % (m - 1);
    q = (r - i + (m - 1)) % (m - 1);
  }
  if (p > q) {
    int x = p;
    p = q;
    q = x;
  }
}

// Cyclic Jacobi on the Hermitian d x d matrix A (shared memory): A becomes
// diagonal (the eigenvalues), U (global) the eigenvectors, A_in = U A U^dagger.
// Scratch: rot / ph (np each), pq (2 np), red_off / red_diag (kThreads each).
__device__ void herm_jacobi(double2* A, double2* U, int d, double2* rot, double2* ph, int* pq,
                            double* red_off, double* red_diag) {
  const int m = d + (d & 1);
  const int np = m / 2;
  for (int e = threadIdx.x; e < d * d; e += kThreads) U[e] = make_double2((e % d) == (e / d) ? 1.0 : 0.0, 0.0);
  __syncthreads();
  for (int sweep = 0; sweep < 40; ++sweep) {
    double off = 0.0, dg = 0.0;
    for (int e = threadIdx.x; e < d * d; e += kThreads) {
      const double v = A[e].x * A[e].x + A[e].y * A[e].y;
      if (e % d == e / d)
        dg += v;
      else
        off += v;
    }
    red_off[threadIdx.x] = off;
    red_diag[threadIdx.x] = dg;
    __syncthreads();
    for (int s = kThreads / 2; s > 0; s >>= 1) {
      if (threadIdx.x < s) {
        red_off[threadIdx.x] += red_off[threadIdx.x + s];
        red_diag[threadIdx.x] += red_diag[threadIdx.x + s];
      }
      __syncthreads();
    }
    const double toff = red_off[0], tdiag = red_diag[0];
    __syncthreads();
    if (!(toff > 1e-30 * tdiag) || toff == 0.0) break;
    for (int r = 0; r < m - 1; ++r) {
      for (int i = threadIdx.x; i < np; i += kThreads) {
        int p, q;
        rr_pair(m, r, i, p, q);
        double c = 1.0, s = 0.0;
        double2 e = make_double2(1.0, 0.0);
        if (q < d) {
          const double2 apq = A[p + d * q];
          const double ab = hypot(apq.x, apq.y);
          if (ab > 0.0) {
            e = make_double2(apq.x / ab, apq.y / ab);
            const double theta = 0.5 * atan2(2.0 * ab, A[q + d * q].x - A[p + d * p].x);
            c = cos(theta);
            s = sin(theta);
          }
        }
        rot[i] = make_double2(c, s);
        ph[i] = e;
        pq[2 * i] = p;
        pq[2 * i + 1] = q;
      }
      __syncthreads();
      // columns: A <- A G, U <- U G
      for (int idx = threadIdx.x; idx < np * d; idx += kThreads) {
        const int i = idx / d, k = idx % d;
        const int p = pq[2 * i], q = pq[2 * i + 1];
        if (q >= d || rot[i].y == 0.0) continue;
        const double c = rot[i].x, s = rot[i].y;
        const double2 e = ph[i];
        const double2 se = make_double2(s * e.x, s * e.y);    // s*e
        const double2 sce = make_double2(s * e.x, -s * e.y);  // s*conj(e)
        double2 akp = A[k + d * p], akq = A[k + d * q];
        double2 np_ = make_double2(c * akp.x, c * akp.y);
        double2 t2 = cmul(sce, akq);
        np_.x -= t2.x;
        np_.y -= t2.y;
        double2 nq = cmul(se, akp);
        nq.x += c * akq.x;
        nq.y += c * akq.y;
        A[k + d * p] = np_;
        A[k + d * q] = nq;
        double2 ukp = U[k + (int64_t)d * p], ukq = U[k + (int64_t)d * q];
        np_ = make_double2(c * ukp.x, c * ukp.y);
        t2 = cmul(sce, ukq);
        np_.x -= t2.x;
        np_.y -= t2.y;
        nq = cmul(se, ukp);
        nq.x += c * ukq.x;
        nq.y += c * ukq.y;
        U[k + (int64_t)d * p] = np_;
        U[k + (int64_t)d * q] = nq;
      }
      __syncthreads();
      // rows: A <- G^dagger A
      for (int idx = threadIdx.x; idx < np * d; idx += kThreads) {
        const int i = idx / d, k = idx % d;
        const int p = pq[2 * i], q = pq[2 * i + 1];
        if (q >= d || rot[i].y == 0.0) continue;
        const double c = rot[i].x, s = rot[i].y;
        const double2 e = ph[i];
        const double2 se = make_double2(s * e.x, s * e.y);
        const double2 sce = make_double2(s * e.x, -s * e.y);
        const double2 apk = A[p + d * k], aqk = A[q + d * k];
        double2 np_ = make_double2(c * apk.x, c * apk.y);
        double2 t2 = cmul(se, aqk);
        np_.x -= t2.x;
        np_.y -= t2.y;
        double2 nq = cmul(sce, apk);
        nq.x += c * aqk.x;
        nq.y += c * aqk.y;
        A[p + d * k] = np_;
        A[q + d * k] = nq;
      }
      __syncthreads();
      for (int i = threadIdx.x; i < np; i += kThreads) {
        const int p = pq[2 * i], q = pq[2 * i + 1];
        if (q < d && rot[i].y != 0.0) {
          A[p + d * q] = cz();
          A[q + d * p] = cz();
        }
      }
      __syncthreads();
    }
  }
}

__device__ __forceinline__ void eig_body(const EigTask& t, double eps) {
  extern __shared__ double2 smem[];
  const int d = t.d;
  const int m = d + (d & 1);
  const int np = m / 2;
  double2* A = smem;                      // d*d
  double2* rot = A + (int64_t)d * d;      // np entries: (c, s)
  double2* ph = rot + np;                 // np entries: e
  double2* fw = ph + np;                  // m entries: f(eigenvalue) in .x
  int* pq = (int*)(fw + m);               // 2*np
  __shared__ double red_off[kThreads], red_diag[kThreads];
  double2* U = t.U;
  for (int e = threadIdx.x; e < d * d; e += kThreads) {
    const int i = e % d, j = e / d;
    const double2 aij = t.rho[i + (int64_t)d * j], aji = t.rho[j + (int64_t)d * i];
    // Hermitian part
    A[e] = (i == j) ? make_double2(aij.x, 0.0)
                    : make_double2(0.5 * (aij.x + aji.x), 0.5 * (aij.y - aji.y));
    // shifted copy for the positive-definiteness certificate below
    U[e] = (i == j) ? make_double2(A[e].x - 100.0 * eps, 0.0) : A[e];
  }
  __syncthreads();
  // Fast path.  If every eigenvalue exceeds 50*eps, eps*exp(-w/eps) changes
  // 1/w by less than 4e-24 relative, so the regularised inverse is the plain
  // inverse.  A Cholesky factorisation of rho - 100*eps*I that succeeds
  // certifies that bound (its backward error, ~d*2^-53*|rho|, is far below
  // 50*eps for eps = 1e-10 and normalised states); then rho^-1 comes from a
  // Gauss-Jordan inversion (no pivoting needed for a positive definite
  // matrix) in O(d^3) instead of a Jacobi eigensolver.
  __shared__ int not_pd;
  __shared__ double2 piv_s;
  if (threadIdx.x == 0) not_pd = 0;
  __syncthreads();
  for (int k = 0; k < d; ++k) {
    const double dk = U[k + (int64_t)d * k].x;
    if (!(dk > 0.0)) {
      if (threadIdx.x == 0) not_pd = 1;
      break;  // uniform: every thread reads the same value
    }
    const double l = sqrt(dk);
    __syncthreads();
    for (int i = k + threadIdx.x; i < d; i += kThreads) {
      double2 v = U[i + (int64_t)d * k];
      U[i + (int64_t)d * k] = make_double2(v.x / l, v.y / l);
    }
    __syncthreads();
    // trailing update of the lower triangle: U(i,j) -= L(i,k) conj(L(j,k))
    const int rem = d - k - 1;
    for (int e = threadIdx.x; e < rem * rem; e += kThreads) {
      const int i = k + 1 + e % rem, j = k + 1 + e / rem;
      if (j > i) continue;
      const double2 li = U[i + (int64_t)d * k], lj = U[j + (int64_t)d * k];
      double2 u = U[i + (int64_t)d * j];
      cfma(u, make_double2(-li.x, -li.y), make_double2(lj.x, -lj.y));
      U[i + (int64_t)d * j] = u;
    }
    __syncthreads();
  }
  __syncthreads();
  if (!not_pd) {
    double2* X = t.rhoinv;
    for (int e = threadIdx.x; e < d * d; e += kThreads)
      X[e] = make_double2((e % d) == (e / d) ? 1.0 : 0.0, 0.0);
    __syncthreads();
    for (int col = 0; col < d; ++col) {
      if (threadIdx.x == 0) {
        const double2 v = A[col + d * col];
        const double den = v.x * v.x + v.y * v.y;
        piv_s = make_double2(v.x / den, -v.y / den);
      }
      __syncthreads();
      const double2 pinv = piv_s;
      for (int j = threadIdx.x; j < d; j += kThreads) {
        A[col + d * j] = cmul(A[col + d * j], pinv);
        X[col + (int64_t)d * j] = cmul(X[col + (int64_t)d * j], pinv);
      }
      __syncthreads();
      // column col of A before elimination (fw reused as the factor column)
      for (int r = threadIdx.x; r < d; r += kThreads) fw[r] = A[r + d * col];
      __syncthreads();
      for (int e = threadIdx.x; e < d * d; e += kThreads) {
        const int r = e % d, j = e / d;
        if (r == col) continue;
        const double2 f = fw[r];
        double2 a = A[e], x = X[e];
        cfma(a, make_double2(-f.x, -f.y), A[col + d * j]);
        cfma(x, make_double2(-f.x, -f.y), X[col + (int64_t)d * j]);
        A[e] = a;
        X[e] = x;
      }
      __syncthreads();
    }
    return;
  }
  herm_jacobi(A, U, d, rot, ph, pq, red_off, red_diag);
  for (int i = threadIdx.x; i < d; i += kThreads) {
    const double w = A[i + d * i].x;
    fw[i].x = 1.0 / (w + eps * exp(-w / eps));
  }
  __syncthreads();
  for (int e = threadIdx.x; e < d * d; e += kThreads) {
    const int i = e % d, j = e / d;
    double2 acc = cz();
    for (int k = 0; k < d; ++k) {
      const double2 uik = U[i + (int64_t)d * k];
      const double2 ujk = U[j + (int64_t)d * k];
      const double f = fw[k].x;
      // acc += uik * f * conj(ujk)
      cfma(acc, make_double2(uik.x * f, uik.y * f), make_double2(ujk.x, -ujk.y));
    }
    t.rhoinv[e] = acc;
  }
}

__global__ void __launch_bounds__(kThreads) k_eig(const EigTask* __restrict__ tasks, int64_t task0,
                                                  double eps) {
  const EigTask t = tasks[task0 + blockIdx.x];
  eig_body(t, eps);
}

// ---------------------------------------------------------------------------
// Projector pieces of LayerDerivative (projectOut + rho^-1), per node:
//   Sinv = S^-1 (Gauss-Jordan, partial pivoting; S is overwritten)
//   P    = Sinv D
//   M2   = -(rhoinv P^T)
// so that the derivative is dPsi = alpha ((H Phi) rhoinv^T + Phi M2^T).
// ---------------------------------------------------------------------------
// Projector of one node in the arithmetic of the plan: X = S^-1 by
// Gauss-Jordan with partial pivoting (warp-parallel pivot search), then
// P = X D and M2 = -rhoinv P^T.  S and X live in shared memory when
// 2 d^2 elements fit (smem != 0), else in the task's Sinv / P slots.
template <class P>
__global__ void __launch_bounds__(kThreads) k_proj2(const ProjTask* __restrict__ tasks, int64_t task0, int smem) {
  typedef typename P::S S;
  typedef typename P::A A;
  extern __shared__ __align__(16) unsigned char proj_smem[];
  const ProjTask t = tasks[task0 + blockIdx.x];
  const int d = t.d;
  S* W = smem ? reinterpret_cast<S*>(proj_smem) : reinterpret_cast<S*>(t.P);      // working S
  S* X = smem ? W + d * d : reinterpret_cast<S*>(t.Sinv);                          // becomes S^-1
  __shared__ S fcol[kHpMaxDim];
  __shared__ int piv;
  __shared__ S pinv;
  const S* Sin = reinterpret_cast<const S*>(t.S);
  for (int e = threadIdx.x; e < d * d; e += kThreads) {
    W[e] = Sin[e];
    S z = P::zero();
    if ((e % d) == (e / d)) z = P::coef(make_double2(1.0, 0.0));
    X[e] = z;
  }
  __syncthreads();
  for (int col = 0; col < d; ++col) {
    if (threadIdx.x < 32) {  // pivot: largest |S(r, col)|, r >= col
      double bv = -1.0;
      int best = col;
      for (int r = col + threadIdx.x; r < d; r += 32) {
        const double m = P::mag2(W[r + d * col]);
        if (m > bv) bv = m, best = r;
      }
      for (int off = 16; off > 0; off >>= 1) {
        const double ov = __shfl_down_sync(0xffffffffu, bv, off);
        const int ob = __shfl_down_sync(0xffffffffu, best, off);
        if (ov > bv || (ov == bv && ob < best)) bv = ov, best = ob;
      }
      if (threadIdx.x == 0) piv = best;
    }
    __syncthreads();
    const int pr = piv;
    if (pr != col) {
      for (int j = threadIdx.x; j < d; j += kThreads) {
        S x = W[col + d * j];
        W[col + d * j] = W[pr + d * j];
        W[pr + d * j] = x;
        x = X[col + d * j];
        X[col + d * j] = X[pr + d * j];
        X[pr + d * j] = x;
      }
    }
    __syncthreads();
    if (threadIdx.x == 0) pinv = P::recip(W[col + d * col]);
    __syncthreads();
    const S pv = pinv;
    for (int j = threadIdx.x; j < d; j += kThreads) {
      W[col + d * j] = P::mul(W[col + d * j], pv);
      X[col + d * j] = P::mul(X[col + d * j], pv);
    }
    __syncthreads();
    for (int r = threadIdx.x; r < d; r += kThreads) fcol[r] = P::neg(W[r + d * col]);
    __syncthreads();
    for (int e = threadIdx.x; e < d * d; e += kThreads) {
      const int r = e % d, j = e / d;
      if (r == col) continue;
      const S f = fcol[r];
      if (j > col) {
        A w = W[e];
        P::mac(w, f, W[col + d * j]);
        W[e] = P::fin(w);
      }
      A x = X[e];
      P::mac(x, f, X[col + d * j]);
      X[e] = P::fin(x);
    }
    __syncthreads();
  }
  // P = X D into W (S is no longer needed)
  const S* D = reinterpret_cast<const S*>(t.D);
  for (int e = threadIdx.x; e < d * d; e += kThreads) {
    const int i = e % d, j = e / d;
    A acc = P::zero();
    for (int k = 0; k < d; ++k) {
      P::mac(acc, X[i + d * k], D[k + d * j]);
      if (k & 1) P::norm(acc);
    }
    W[e] = P::fin(acc);
  }
  __syncthreads();
  // M2 = -rhoinv P^T
  const S* Ri = reinterpret_cast<const S*>(t.rhoinv);
  S* M2 = reinterpret_cast<S*>(t.M2);
  for (int e = threadIdx.x; e < d * d; e += kThreads) {
    const int j = e % d, m = e / d;
    A acc = P::zero();
    for (int k = 0; k < d; ++k) {
      P::mac(acc, Ri[j + d * k], W[m + d * k]);
      if (k & 1) P::norm(acc);
    }
    M2[e] = P::neg(P::fin(acc));
  }
}

__global__ void k_identity(double2* m, int d, int prec) {
  for (int e = threadIdx.x; e < d * d; e += blockDim.x) {
    const bool diag = (e % d) == (e / d);
    if (prec >= 1)
      reinterpret_cast<float4*>(m)[e] = make_float4(diag ? 1.f : 0.f, 0.f, 0.f, 0.f);
    else
      m[e] = make_double2(diag ? 1.0 : 0.0, 0.0);
  }
}

// Eight independent FMA chains per thread; one store per thread keeps the
// chains live.  Every store index is < gridDim.x * blockDim.x.
__global__ void __launch_bounds__(kThreads) k_fp64_fma(double* out, int iters, double a, double b) {
  double acc[8];
#pragma unroll
  for (int i = 0; i < 8; ++i) acc[i] = threadIdx.x + i;
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int i = 0; i < 8; ++i) acc[i] = fma(acc[i], a, b);
  }
  double s = 0;
#pragma unroll
  for (int i = 0; i < 8; ++i) s += acc[i];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

// The double-float complex multiply-add of the chain kernels (DF64::mac,
// renormalised every second step) on eight register accumulators per thread:
// the ceiling of double-float arithmetic on this GPU, no memory traffic.
// Every product reads another accumulator (acc[i] += a * acc[i ^ 4]), so
// nothing is loop-invariant; |a| = 1e-3 keeps the values finite.  One store
// per thread, index < gridDim.x * blockDim.x.
__global__ void __launch_bounds__(kThreads) k_df64_mac(float4* out, int iters, float4 a, float4 b) {
  float4 acc[8];
#pragma unroll
  for (int i = 0; i < 8; ++i) acc[i] = make_float4(threadIdx.x + i, 0.f, b.x * i, 0.f);
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      DF64::mac(acc[i], a, acc[i ^ 4]);
      if (it & 1) DF64::norm(acc[i]);
    }
  }
  float4 s = acc[0];
#pragma unroll
  for (int i = 1; i < 8; ++i) s = DF64::plus(s, acc[i]);
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

inline int64_t eig_smem_bytes(int d) {
  const int m = d + (d & 1);
  const int np = m / 2;
  return 16 * ((int64_t)d * d + 2 * np + m) + 8 * (int64_t)np + 16;
}

__global__ void __launch_bounds__(kThreads) k_axpy(double2* out, const double2* x, double2 a,
                                                   const double2* y, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * kThreads + threadIdx.x; i < n; i += (int64_t)gridDim.x * kThreads) {
    double2 v = x[i];
    cfma(v, a, y[i]);
    out[i] = v;
  }
}
}  // namespace

// ---------------------------------------------------------------------------
// Krylov vector helpers of the SCF sweep (complex128).
// k_dot: out = sum_i conj(a_i) b_i in one block; every thread sums a fixed
// strided subset in order, then a fixed-order tree in shared memory, so the
// result is reproducible run to run.
// k_lincomb: out_i = sum_t c_t v_t,i over up to kLinCombMax vectors.
// ---------------------------------------------------------------------------
constexpr int kDotThreads = 512;
constexpr int64_t kDotParts = 256;

__global__ void __launch_bounds__(kDotThreads) k_dot(const double2* __restrict__ a,
                                                     const double2* __restrict__ b, int64_t n,
                                                     double2* __restrict__ out) {
  __shared__ double2 red[kDotThreads];
  double2 acc = cz();
  for (int64_t i = threadIdx.x; i < n; i += kDotThreads) {
    if (b)
      cfmac(acc, a[i], b[i]);
    else
      acc = cadd(acc, a[i]);
  }
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int w = kDotThreads / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) red[threadIdx.x] = cadd(red[threadIdx.x], red[threadIdx.x + w]);
    __syncthreads();
  }
  if (threadIdx.x == 0) out[0] = red[0];
}

__global__ void __launch_bounds__(kThreads) k_lincomb(double2* __restrict__ out, LinComb lc, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * kThreads + threadIdx.x; i < n; i += (int64_t)gridDim.x * kThreads) {
    double2 acc = cz();
    for (int t = 0; t < lc.count; ++t) cfma(acc, lc.c[t], lc.v[t][i]);
    out[i] = acc;
  }
}

// first pass: block b sums its contiguous slice in a fixed order
__global__ void __launch_bounds__(kDotThreads) k_dot_part(const double2* __restrict__ a,
                                                          const double2* __restrict__ b, int64_t n,
                                                          int64_t slice, double2* __restrict__ part) {
  __shared__ double2 red[kDotThreads];
  const int64_t lo = (int64_t)blockIdx.x * slice, hi = min(n, lo + slice);
  double2 acc = cz();
  for (int64_t i = lo + threadIdx.x; i < hi; i += kDotThreads) cfmac(acc, a[i], b[i]);
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int w = kDotThreads / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) red[threadIdx.x] = cadd(red[threadIdx.x], red[threadIdx.x + w]);
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}

// complex128 <-> double-float copy of n elements (dir 0: to double-float)
__global__ void __launch_bounds__(kThreads) k_convert(void* __restrict__ dst, const void* __restrict__ src,
                                                      int64_t n, int dir) {
  for (int64_t i = (int64_t)blockIdx.x * kThreads + threadIdx.x; i < n; i += (int64_t)gridDim.x * kThreads) {
    if (dir == 0) {
      const double2 v = reinterpret_cast<const double2*>(src)[i];
      const float2 r = df_split(v.x), m = df_split(v.y);
      reinterpret_cast<float4*>(dst)[i] = make_float4(r.x, r.y, m.x, m.y);
    } else {
      const float4 v = reinterpret_cast<const float4*>(src)[i];
      reinterpret_cast<double2*>(dst)[i] = make_double2((double)v.x + (double)v.y, (double)v.z + (double)v.w);
    }
  }
}

cudaError_t launch_convert(void* dst, const void* src, int64_t n, int dir, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  const int blocks = (int)std::min<int64_t>((n + kThreads - 1) / kThreads, 152 * 8);
  k_convert<<<blocks, kThreads, 0, s>>>(dst, src, n, dir);
  return cudaGetLastError();
}

cudaError_t launch_dot(const double2* a, const double2* b, int64_t n, double2* out, cudaStream_t s) {
  // slices of >= 8192 elements, at most kDotParts of them; the partial sums
  // go to out[1 ..] and are added in order by one block into out[0]
  int64_t parts = std::min<int64_t>(kDotParts, std::max<int64_t>(1, (n + 8191) / 8192));
  const int64_t slice = (n + parts - 1) / parts;
  parts = std::max<int64_t>(1, (n + slice - 1) / slice);
  k_dot_part<<<(unsigned)parts, kDotThreads, 0, s>>>(a, b, n, slice, out + 1);
  k_dot<<<1, kDotThreads, 0, s>>>(out + 1, nullptr, parts, out);
  return cudaGetLastError();
}

cudaError_t launch_hp_one_shape(const HPTask& t, int ntiles, double2* ws, cudaStream_t s);

cudaError_t launch_hp_split(const HPTask& task, double2* ws, int64_t ws_elems, cudaStream_t s) {
  HPTask t = task;
  const int aB = t.aB > 0 ? t.aB : t.a;
  if (t.a > kHpMaxDim || aB > kHpMaxDim || t.a < 1 || aB < 1) return cudaErrorInvalidValue;
  hp_shape(std::min(std::max(t.a, aB), kHpTile), &t.rows, &t.cols);
  const int ntiles = ((t.a + kHpTile - 1) / kHpTile) * ((aB + kHpTile - 1) / kHpTile);
  const int64_t K = (int64_t)t.before * t.after;
  int64_t kc = std::max<int64_t>(256, (K * ntiles + 4 * 152 - 1) / (4 * 152));
  kc = (kc + kHpRows - 1) / kHpRows * kHpRows;
  int64_t splits = (K + kc - 1) / kc;
  const int64_t per = (int64_t)t.a * aB;
  if (splits > 1 && splits * per > ws_elems) {  // fewer, longer ranges to fit the workspace
    splits = std::max<int64_t>(1, ws_elems / per);
    kc = (K + splits - 1) / splits;
    splits = (K + kc - 1) / kc;
  }
  t.splits = (int)splits;
  t.kchunk = (int)std::min<int64_t>(K, kc);
  t.ws = 0;
  cudaError_t e = launch_hp_one_shape(t, ntiles, ws, s);
  if (e != cudaSuccess) return e;
  if (t.splits > 1) k_hp_sum_one<F64><<<(unsigned)std::min<int64_t>(64, (per + kThreads - 1) / kThreads), kThreads, 0, s>>>(t, ws);
  return cudaGetLastError();
}

cudaError_t launch_lincomb(double2* out, const LinComb& lc, int64_t n, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  if (lc.count < 0 || lc.count > kLinCombMax) return cudaErrorInvalidValue;
  const int64_t want = (n + kThreads - 1) / kThreads;
  const int blocks = (int)std::min<int64_t>(want, 152 * 8);
  k_lincomb<<<blocks, kThreads, 0, s>>>(out, lc, n);
  return cudaGetLastError();
}

cudaError_t launch_axpy(double2* out, const double2* x, double2 a, const double2* y, int64_t n,
                        cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int64_t want = (n + kThreads - 1) / kThreads;
  const int blocks = (int)std::min<int64_t>(want, (int64_t)sms * 8);
  k_axpy<<<blocks, kThreads, 0, s>>>(out, x, a, y, n);
  return cudaGetLastError();
}

cudaError_t probe_df64_peak(cudaStream_t s, double* tflops) {
  int dev = 0, sms = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return e;
  const int blocks = sms * 8, iters = 2048;
  float4* buf = nullptr;
  e = cudaMallocAsync((void**)&buf, sizeof(float4) * blocks * kThreads, s);
  if (e != cudaSuccess) return e;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  const float4 a = make_float4(1e-3f, 1e-11f, 2e-4f, -1e-12f), b = make_float4(0.5f, 0.f, 0.f, 0.f);
  k_df64_mac<<<blocks, kThreads, 0, s>>>(buf, iters, a, b);  // warm-up
  cudaEventRecord(e0, s);
  k_df64_mac<<<blocks, kThreads, 0, s>>>(buf, iters, a, b);
  cudaEventRecord(e1, s);
  e = cudaEventSynchronize(e1);
  float ms = 0;
  if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFreeAsync(buf, s);
  cudaStreamSynchronize(s);
  if (e != cudaSuccess) return e;
  // 8 flops (complex128-equivalent) per complex multiply-add
  *tflops = 8.0 * 8.0 * iters * (double)blocks * kThreads / (ms * 1e-3) / 1e12;
  return cudaGetLastError();
}

cudaError_t probe_fp64_peak(cudaStream_t s, double* tflops) {
  int dev = 0, sms = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return e;
  const int blocks = sms * 8, iters = 4096;
  double* buf = nullptr;
  e = cudaMallocAsync((void**)&buf, sizeof(double) * blocks * kThreads, s);
  if (e != cudaSuccess) return e;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  k_fp64_fma<<<blocks, kThreads, 0, s>>>(buf, iters, 0.999, 0.001);  // warm-up
  cudaEventRecord(e0, s);
  k_fp64_fma<<<blocks, kThreads, 0, s>>>(buf, iters, 0.999, 0.001);
  cudaEventRecord(e1, s);
  e = cudaEventSynchronize(e1);
  float ms = 0;
  if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFreeAsync(buf, s);
  cudaStreamSynchronize(s);
  if (e != cudaSuccess) return e;
  *tflops = 2.0 * 8.0 * iters * (double)blocks * kThreads / (ms * 1e-3) / 1e12;
  return cudaGetLastError();
}

template <class P, int R, int C>
cudaError_t launch_hp_rc(const HPTask* tasks, const int4* tiles, int64_t first, int64_t n,
                         typename P::S* ws, cudaStream_t s) {
  cudaError_t e = cudaFuncSetAttribute(k_hp<P, R, C>, cudaFuncAttributeMaxDynamicSharedMemorySize, kHpSmem);
  if (e != cudaSuccess) return e;
  k_hp<P, R, C><<<(unsigned)n, kThreads, kHpSmem, s>>>(tasks, tiles, first, ws);
  return cudaSuccess;
}

// the micro-tile shapes the planner chooses (rows x cols of outputs per thread)
template <class P>
cudaError_t launch_hp_shape(int rows, int cols, const HPTask* tasks, const int4* tiles, int64_t first,
                            int64_t n, typename P::S* ws, cudaStream_t s) {
  switch (rows * 8 + cols) {
    case 1 * 8 + 1: return launch_hp_rc<P, 1, 1>(tasks, tiles, first, n, ws, s);
    case 1 * 8 + 2: return launch_hp_rc<P, 1, 2>(tasks, tiles, first, n, ws, s);
    case 1 * 8 + 3: return launch_hp_rc<P, 1, 3>(tasks, tiles, first, n, ws, s);
    case 1 * 8 + 4: return launch_hp_rc<P, 1, 4>(tasks, tiles, first, n, ws, s);
    case 2 * 8 + 3: return launch_hp_rc<P, 2, 3>(tasks, tiles, first, n, ws, s);
    case 2 * 8 + 4: return launch_hp_rc<P, 2, 4>(tasks, tiles, first, n, ws, s);
    case 3 * 8 + 3: return launch_hp_rc<P, 3, 3>(tasks, tiles, first, n, ws, s);
    case 3 * 8 + 4: return launch_hp_rc<P, 3, 4>(tasks, tiles, first, n, ws, s);
    case 4 * 8 + 4: return launch_hp_rc<P, 4, 4>(tasks, tiles, first, n, ws, s);
    default: return cudaErrorInvalidValue;
  }
}

template <int R, int C>
cudaError_t launch_hp_one_rc(const HPTask& t, int ntiles, double2* ws, cudaStream_t s) {
  cudaError_t e = cudaFuncSetAttribute(k_hp_one<F64, R, C>, cudaFuncAttributeMaxDynamicSharedMemorySize, kHpSmem);
  if (e != cudaSuccess) return e;
  k_hp_one<F64, R, C><<<(unsigned)((int64_t)ntiles * t.splits), kThreads, kHpSmem, s>>>(t, ntiles, ws);
  return cudaSuccess;
}

cudaError_t launch_hp_one_shape(const HPTask& t, int ntiles, double2* ws, cudaStream_t s) {
  switch (t.rows * 8 + t.cols) {
    case 1 * 8 + 1: return launch_hp_one_rc<1, 1>(t, ntiles, ws, s);
    case 1 * 8 + 2: return launch_hp_one_rc<1, 2>(t, ntiles, ws, s);
    case 1 * 8 + 3: return launch_hp_one_rc<1, 3>(t, ntiles, ws, s);
    case 1 * 8 + 4: return launch_hp_one_rc<1, 4>(t, ntiles, ws, s);
    case 2 * 8 + 3: return launch_hp_one_rc<2, 3>(t, ntiles, ws, s);
    case 2 * 8 + 4: return launch_hp_one_rc<2, 4>(t, ntiles, ws, s);
    case 3 * 8 + 3: return launch_hp_one_rc<3, 3>(t, ntiles, ws, s);
    case 3 * 8 + 4: return launch_hp_one_rc<3, 4>(t, ntiles, ws, s);
    case 4 * 8 + 4: return launch_hp_one_rc<4, 4>(t, ntiles, ws, s);
    default: return cudaErrorInvalidValue;
  }
}


// ---------------------------------------------------------------------------
// CDVR kernels (complex128)
// ---------------------------------------------------------------------------
// Strided complex contraction (TCTask): one block per 32 x 32 output tile,
// k in chunks of 16 staged through shared memory.  Operand tiles are read
// along whichever of their two indices has unit stride.
constexpr int kTcK = 16;
__global__ void __launch_bounds__(kThreads) k_tc(const TCTask* __restrict__ tasks,
                                                 const int4* __restrict__ tiles, int64_t tile0) {
  const int4 tl = tiles[tile0 + blockIdx.x];
  const TCTask t = tasks[tl.x];
  const int64_t M = (int64_t)t.M0 * t.M1, N = (int64_t)t.N0 * t.N1, K = (int64_t)t.K0 * t.K1;
  const int64_t mb = (int64_t)tl.y * kTcTile, nb = (int64_t)tl.z * kTcTile;
  __shared__ double2 As[kTcK][kTcTile + 1];
  __shared__ double2 Bs[kTcK][kTcTile + 1];
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  double2 acc[2][2];
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 2; ++j) acc[i][j] = cz();
  const bool a_mfast = t.am0 == 1 || t.M0 * (int64_t)t.M1 == 1;
  const bool b_nfast = t.bn0 == 1 || t.N0 * (int64_t)t.N1 == 1;
  for (int64_t k0 = 0; k0 < K; k0 += kTcK) {
#pragma unroll
    for (int r = 0; r < 2; ++r) {
      const int e = threadIdx.x + r * kThreads;  // 512 elements of each tile
      int mi, ki;
      if (a_mfast) {
        mi = e & 31;
        ki = e >> 5;
      } else {
        ki = e & 15;
        mi = e >> 4;
      }
      const int64_t m = mb + mi, k = k0 + ki;
      double2 v = cz();
      if (m < M && k < K) {
        const int64_t m0 = m % t.M0, m1 = m / t.M0, kk0 = k % t.K0, kk1 = k / t.K0;
        v = t.A[m0 * t.am0 + m1 * t.am1 + kk0 * t.ak0 + kk1 * t.ak1];
        if (t.conjA) v.y = -v.y;
      }
      As[ki][mi] = v;
      int ni, kj;
      if (b_nfast) {
        ni = e & 31;
        kj = e >> 5;
      } else {
        kj = e & 15;
        ni = e >> 4;
      }
      const int64_t nn = nb + ni, kb = k0 + kj;
      double2 w = cz();
      if (nn < N && kb < K) {
        const int64_t n0 = nn % t.N0, n1 = nn / t.N0, kk0 = kb % t.K0, kk1 = kb / t.K0;
        w = t.B[kk0 * t.bk0 + kk1 * t.bk1 + n0 * t.bn0 + n1 * t.bn1];
        if (t.conjB) w.y = -w.y;
      }
      Bs[kj][ni] = w;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < kTcK; ++kk) {
      const double2 a0 = As[kk][ty * 2], a1 = As[kk][ty * 2 + 1];
      const double2 b0 = Bs[kk][tx * 2], b1 = Bs[kk][tx * 2 + 1];
      cfma(acc[0][0], a0, b0);
      cfma(acc[0][1], a0, b1);
      cfma(acc[1][0], a1, b0);
      cfma(acc[1][1], a1, b1);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 2; ++j) {
      const int64_t m = mb + ty * 2 + i, nn = nb + tx * 2 + j;
      if (m >= M || nn >= N) continue;
      const int64_t off = (m % t.M0) * t.cm0 + (m / t.M0) * t.cm1 + (nn % t.N0) * t.cn0 + (nn / t.N0) * t.cn1;
      const double2 v = cmul(t.alpha, acc[i][j]);
      if (t.add) {
        const double2 o = t.C[off];
        t.C[off] = make_double2(o.x + v.x, o.y + v.y);
      } else {
        t.C[off] = v;
      }
    }
}

__device__ double2 block_sum2(double2 v, double2* red) {
  red[threadIdx.x] = v;
  __syncthreads();
  for (int s = kThreads / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) {
      red[threadIdx.x].x += red[threadIdx.x + s].x;
      red[threadIdx.x].y += red[threadIdx.x + s].y;
    }
    __syncthreads();
  }
  const double2 r = red[0];
  __syncthreads();
  return r;
}

// out = gramSchmidt(in + noise) (include/Core/Tensor_Implementation.h:805-853):
// per column, up to 15 passes of projection on the previous columns and
// normalisation, while the summed |overlap| of a pass exceeds 1e-12.
__global__ void __launch_bounds__(kThreads) k_gs(const GSTask* __restrict__ tasks, int64_t task0) {
  const GSTask t = tasks[task0 + blockIdx.x];
  __shared__ double2 red[kThreads];
  const int64_t rows = t.rows;
  const int64_t tot = rows * t.cols;
  for (int64_t e = threadIdx.x; e < tot; e += kThreads) {
    const double2 a = t.in[e], z = t.noise[e];
    t.out[e] = make_double2(a.x + z.x, a.y + z.y);
  }
  __syncthreads();
  double2* A = t.out;
  for (int n = 0; n < t.cols; ++n) {
    double2* an = A + rows * n;
    for (int iter = 0; iter < 15; ++iter) {
      double accum = 0;
      for (int m = 0; m < n; ++m) {
        const double2* am = A + rows * m;
        double2 part = cz();
        for (int64_t i = threadIdx.x; i < rows; i += kThreads) cfmac(part, am[i], an[i]);
        const double2 ov = block_sum2(part, red);
        accum += sqrt(ov.x * ov.x + ov.y * ov.y);
        for (int64_t i = threadIdx.x; i < rows; i += kThreads) {
          const double2 x = cmul(ov, am[i]);
          an[i] = make_double2(an[i].x - x.x, an[i].y - x.y);
        }
        __syncthreads();
      }
      double2 part = cz();
      for (int64_t i = threadIdx.x; i < rows; i += kThreads) part.x += an[i].x * an[i].x + an[i].y * an[i].y;
      const double nrm = block_sum2(part, red).x;
      if (nrm != 0.0) {
        const double sc = sqrt(nrm);
        for (int64_t i = threadIdx.x; i < rows; i += kThreads) an[i] = make_double2(an[i].x / sc, an[i].y / sc);
      }
      __syncthreads();
      if (!(accum > 1e-12)) break;
    }
  }
}

inline int64_t eigf_smem_bytes(int d) { return eig_smem_bytes(d) + 4 * (int64_t)(d + 1) + 16; }

// spectral functions of a Hermitian matrix (EigFTask)
__global__ void __launch_bounds__(kThreads) k_eigf(const EigFTask* __restrict__ tasks, int64_t task0) {
  extern __shared__ double2 smem[];
  const EigFTask t = tasks[task0 + blockIdx.x];
  const int d = t.d;
  const int m = d + (d & 1);
  const int np = m / 2;
  double2* A = smem;
  double2* rot = A + (int64_t)d * d;
  double2* ph = rot + np;
  double2* fw = ph + np;
  int* pq = (int*)(fw + m);
  int* perm = pq + 2 * np;
  __shared__ double red_off[kThreads], red_diag[kThreads];
  for (int e = threadIdx.x; e < d * d; e += kThreads) {
    const int i = e % d, j = e / d;
    const double2 aij = t.A[i + (int64_t)d * j], aji = t.A[j + (int64_t)d * i];
    A[e] = (i == j) ? make_double2(aij.x, 0.0) : make_double2(0.5 * (aij.x + aji.x), 0.5 * (aij.y - aji.y));
  }
  __syncthreads();
  herm_jacobi(A, t.U, d, rot, ph, pq, red_off, red_diag);
  __syncthreads();
  const double2* U = t.U;
  if (t.fn == 4) {
    if (threadIdx.x == 0) {  // ascending order of the eigenvalues
      for (int i = 0; i < d; ++i) perm[i] = i;
      for (int i = 0; i < d; ++i) {
        int best = i;
        for (int j = i + 1; j < d; ++j)
          if (A[perm[j] + d * perm[j]].x < A[perm[best] + d * perm[best]].x) best = j;
        const int x = perm[i];
        perm[i] = perm[best];
        perm[best] = x;
      }
    }
    __syncthreads();
    for (int e = threadIdx.x; e < d * d; e += kThreads) {
      const int i = e % d, j = e / d;
      const double2 u = U[j + (int64_t)d * perm[i]];
      t.out[e] = make_double2(u.x, -u.y);
    }
    for (int i = threadIdx.x; i < d; i += kThreads) t.vals[i] = make_double2(A[perm[i] + d * perm[i]].x, 0.0);
    return;
  }
  const double eps = t.eps;
  for (int i = threadIdx.x; i < d; i += kThreads) {
    const double w = A[i + d * i].x;
    double f;
    if (t.fn == 0) {
      f = 1.0 / (w + eps * exp(-w / eps));
    } else {
      const double g = sqrt(fmax(w, 0.0));
      if (t.fn == 1)
        f = g;
      else if (t.fn == 2)
        f = 1.0 / (g + eps * exp(-g / eps));
      else
        f = g + eps * exp(-g / eps);
    }
    fw[i].x = f;
  }
  __syncthreads();
  for (int e = threadIdx.x; e < d * d; e += kThreads) {
    const int i = e % d, j = e / d;
    double2 acc = cz();
    for (int k = 0; k < d; ++k) {
      const double2 uik = U[i + (int64_t)d * k];
      const double2 ujk = U[j + (int64_t)d * k];
      const double fk = fw[k].x;
      cfma(acc, make_double2(uik.x * fk, uik.y * fk), make_double2(ujk.x, -ujk.y));
    }
    t.out[e] = acc;
  }
}

// polynomial potential on grid tensors (VPotTask): terms in order, each
// product left to right, nothing fused (the CPU restatement does the same)
__global__ void __launch_bounds__(kThreads) k_vpot(const VPotTask* __restrict__ tasks,
                                                   const VCoord* __restrict__ coords,
                                                   const int2* __restrict__ tiles, int64_t tile0,
                                                   const PotTerm* __restrict__ terms,
                                                   const PotFactor* __restrict__ factors, int n_terms) {
  const int2 tl = tiles[tile0 + blockIdx.x];
  const VPotTask t = tasks[tl.x];
  const int64_t e = (int64_t)tl.y + threadIdx.x;
  if (e >= t.n) return;
  int idx[6];
  int64_t r = e;
#pragma unroll
  for (int k = 0; k < 6; ++k) {
    if (k < t.order) {
      idx[k] = (int)(r % t.dims[k]);
      r /= t.dims[k];
    } else {
      idx[k] = 0;
    }
  }
  double v = 0.0;
  for (int q = 0; q < n_terms; ++q) {
    const PotTerm pt = terms[q];
    double tv = pt.c;
    for (int fct = pt.first; fct < pt.first + pt.count; ++fct) {
      const PotFactor pf = factors[fct];
      const VCoord c = coords[t.first + pf.mode];
      const double x = c.grid[idx[c.index]].x;
      for (int p = 0; p < pf.power; ++p) tv = __dmul_rn(tv, x);
    }
    v = __dadd_rn(v, tv);
  }
  t.out[e] = make_double2(v, 0.0);
}

// local part of the correction tensor (DVLTask)
__global__ void __launch_bounds__(kThreads) k_dvl(const DVLTask* __restrict__ tasks,
                                                  const int2* __restrict__ tiles, int64_t tile0) {
  const int2 tl = tiles[tile0 + blockIdx.x];
  const DVLTask t = tasks[tl.x];
  const int64_t d = t.d;
  const int64_t e = (int64_t)tl.y + threadIdx.x;
  if (e >= d * d * d * d) return;
  const int64_t l1 = e % d, i0 = e / d % d, m1 = e / (d * d) % d, i3 = e / (d * d * d);
  double2 v = cz();
  if (i0 == i3) {
    const int64_t bef = t.bef;
    for (int64_t b = 0; b < bef; ++b) {
      const double2 a = t.cup[b + bef * l1];
      const double2 x = cmul(make_double2(a.x, -a.y), t.vnode[b + bef * i0]);
      cfma(v, x, t.cup[b + bef * m1]);
    }
  }
  if (l1 == m1 && i0 == i3) {
    const double2 ve = t.vedge[l1 + d * i0];
    v = make_double2(v.x - ve.x, v.y - ve.y);
  }
  t.dv[e] = v;
}

// out = (add ? out : 0) + v * in, elementwise (EWTask)
__global__ void __launch_bounds__(kThreads) k_ew(const EWTask* __restrict__ tasks,
                                                 const int2* __restrict__ tiles, int64_t tile0) {
  const int2 tl = tiles[tile0 + blockIdx.x];
  const EWTask t = tasks[tl.x];
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int64_t e = (int64_t)tl.y + threadIdx.x + (int64_t)q * kThreads;
    if (e >= t.n) continue;
    double2 r = cmul(t.v[e], t.in[e]);
    if (t.add) {
      const double2 o = t.out[e];
      r = make_double2(r.x + o.x, r.y + o.y);
    }
    t.out[e] = r;
  }
}

template <class P>
cudaError_t launch_stage_p(const Stage& st, const DevTables& t, double eps, int max_eig_d,
                           cudaStream_t s) {
  switch (st.kind) {
    case ST_MP:
      if (st.n_tiles > 0) k_mp<P><<<(unsigned)st.n_tiles, kThreads, 0, s>>>(t.mp, t.mp_tiles, st.first_tile);
      if (st.noz > 0) {
        cudaError_t e = launch_mp_tc(std::is_same<P, DF64>::value, t.mp, t.mp_oz_tiles, st.oz0, st.noz,
                                     t.mp_oz_tasks, st.ozt0, st.nozt, t.status, s);
        if (e != cudaSuccess) return e;
      }
      break;
    case ST_HP: {
      typedef typename P::S S;
      for (int g = st.seg0; g < st.seg0 + st.nseg; ++g) {
        const int4 sg = t.hp_segs[g];
        cudaError_t e = launch_hp_shape<P>(sg.x, sg.y, t.hp, t.hp_tiles, sg.z, sg.w, reinterpret_cast<S*>(t.hp_ws), s);
        if (e != cudaSuccess) return e;
      }
      if (st.nhti > 0) {
        if (!std::is_same<P, DF64>::value) return cudaErrorInvalidValue;  // the planner emits none
        cudaError_t e = launch_hp_tc(t.hp, t.hp_tc_groups, t.hp_tc_items, st.hti0, st.nhti, t.hp_tc_imgs, st.htu0,
                                     st.nhtu, reinterpret_cast<double2*>(t.hp_ws), t.status, s);
        if (e != cudaSuccess) return e;
      }
      if (st.aux)
        k_hp_sum<P><<<(unsigned)(st.n_tasks * kHpSumChunks), kThreads, 0, s>>>(t.hp, st.first_task,
                                                             reinterpret_cast<const S*>(t.hp_ws));
      break;
    }
    case ST_ACC:
      if (st.n_tiles > 0)
        k_acc<P><<<(unsigned)st.n_tiles, kThreads, 0, s>>>(t.acc, t.acc_terms, t.acc_tiles, st.first_tile);
      if (st.nati > 0) {
        if (!std::is_same<P, DF64>::value) return cudaErrorInvalidValue;  // the planner emits none
        cudaError_t e = launch_acc_tc(t.acc, t.acc_terms, t.acc_tc_items, st.ati0, st.nati, st.atc_units,
                                      t.acc_tc_imgs, st.atu0, st.natu, t.status, s);
        if (e != cudaSuccess) return e;
      }
      break;
    case ST_LIN:
      k_lin<P><<<(unsigned)st.n_tasks, kThreads, 0, s>>>(t.lin, t.lin_terms, st.first_task);
      break;
    case ST_MM:
      k_mm<P><<<(unsigned)st.n_tiles, kThreads, 0, s>>>(t.mm, t.mm_terms, t.mm_tiles, st.first_tile);
      break;
    case ST_EIG: {
      const int64_t sm = eig_smem_bytes(max_eig_d);
      cudaError_t e = cudaFuncSetAttribute(k_eig, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           (int)sm);
      if (e != cudaSuccess) return e;
      k_eig<<<(unsigned)st.n_tasks, kThreads, sm, s>>>(t.eig, st.first_task, eps);
      break;
    }
    case ST_PROJ: {
      // max_eig_d bounds every node's bond
      const int64_t need = 2 * (int64_t)max_eig_d * max_eig_d * 16;
      const int sm = need <= 200 * 1024 ? (int)need : 0;
      if (sm) {
        cudaError_t e = cudaFuncSetAttribute(k_proj2<P>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm);
        if (e != cudaSuccess) return e;
      }
      k_proj2<P><<<(unsigned)st.n_tasks, kThreads, sm, s>>>(t.proj, st.first_task, sm);
      break;
    }
    case ST_CVT:
      k_cvt<<<(unsigned)st.n_tiles, kThreads, 0, s>>>(t.cvt, t.cvt_tiles, st.first_tile);
      break;
    case ST_GRAD:
      k_grad<P><<<(unsigned)st.n_tasks, kThreads, 0, s>>>(t.grad, st.first_task);
      break;
    case ST_TC:
      k_tc<<<(unsigned)st.n_tiles, kThreads, 0, s>>>(t.tc, t.tc_tiles, st.first_tile);
      break;
    case ST_GS:
      k_gs<<<(unsigned)st.n_tasks, kThreads, 0, s>>>(t.gs, st.first_task);
      break;
    case ST_EIGF: {
      const int64_t sm = eigf_smem_bytes(max_eig_d);
      cudaError_t e = cudaFuncSetAttribute(k_eigf, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
      if (e != cudaSuccess) return e;
      k_eigf<<<(unsigned)st.n_tasks, kThreads, sm, s>>>(t.eigf, st.first_task);
      break;
    }
    case ST_WSD:
      return launch_wsd(t.wsd, t.wsd_terms, st.first_task, st.n_tasks, t.wsd_max_n, t.wsd_max_d, s);
    case ST_VPOT:
      k_vpot<<<(unsigned)st.n_tiles, kThreads, 0, s>>>(t.vpot, t.vcoords, t.vpot_tiles, st.first_tile,
                                                       t.pot_terms, t.pot_factors, t.n_pot_terms);
      break;
    case ST_DVL:
      k_dvl<<<(unsigned)st.n_tiles, kThreads, 0, s>>>(t.dvl, t.dvl_tiles, st.first_tile);
      break;
    case ST_EW:
      k_ew<<<(unsigned)st.n_tiles, kThreads, 0, s>>>(t.ew, t.ew_tiles, st.first_tile);
      break;
    default:
      return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

cudaError_t launch_stage(const Stage& st, const DevTables& t, double eps, int max_eig_d,
                         int prec, cudaStream_t s) {
  switch (prec) {
    case 1: return launch_stage_p<DF64>(st, t, eps, max_eig_d, s);
    case 2: return launch_stage_p<C32>(st, t, eps, max_eig_d, s);
    default: return launch_stage_p<F64>(st, t, eps, max_eig_d, s);
  }
}

cudaError_t launch_set_identity(double2* m, int d, int prec, cudaStream_t s) {
  k_identity<<<1, kThreads, 0, s>>>(m, d, prec);
  return cudaGetLastError();
}

cudaError_t launch_single_mp(const MPTask& task, cudaStream_t s, void*) {
  const int64_t slots = (int64_t)task.before * ((task.a_out + 3) / 4) * task.after;
  const int64_t blocks = (slots + kMpTile - 1) / kMpTile;
  if (blocks == 0) return cudaSuccess;
  k_mp_single<<<(unsigned)blocks, kThreads, 0, s>>>(task);
  return cudaGetLastError();
}

cudaError_t launch_single_hp(const HPTask& task, cudaStream_t s, void*) {
  const int aB = task.aB > 0 ? task.aB : task.a;
  const int64_t micro = (int64_t)((task.a + 1) / 2) * ((aB + 1) / 2);
  const int64_t blocks = (micro + kThreads - 1) / kThreads;
  if (blocks == 0) return cudaSuccess;
  const int sm = hp_smem_bytes(task.a, aB);
  if (sm > 200 * 1024) return cudaErrorInvalidValue;
  cudaError_t e = cudaFuncSetAttribute(k_hp_single, cudaFuncAttributeMaxDynamicSharedMemorySize, sm);
  if (e != cudaSuccess) return e;
  k_hp_single<<<(unsigned)blocks, kThreads, sm, s>>>(task);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Allocation-free density inverse.
//
// Callers that may not allocate device memory themselves (code running while
// a CUDA stream is being captured, where cudaMalloc/cudaFree are not
// allowed; latency-critical loops that cannot afford the implicit device
// synchronisation of cudaFree; hosts whose device memory is owned by a pool
// allocator that forbids side allocations) get the regularised inverses of
// density matrices they already hold on the device without handing the
// library any workspace.  The Jacobi eigenvector matrices live in the
// file-scope array below instead of a cudaMalloc'd arena:
//   - capacity kStaticEigElems complex elements (8 MiB): n_mats * d * d
//     must not exceed 524288, e.g. 128 matrices of 64 x 64;
//   - every GPU that loads the library holds these 8 MiB until the process
//     exits;
//   - all calls share the one array and it keeps the last call's contents.
//     The kernel writes every scratch element before reading it (U starts as
//     the identity), so nothing needs clearing between calls; two calls that
//     overlap on the GPU (different streams, contexts or host threads) race
//     on the array and must be ordered by the caller.
// Host code cannot use the array's name as a device address, so the address
// is looked up with cudaGetSymbolAddress (with that device current) on the
// first call that a device sees, and again on the first call after the
// device's context was replaced (cudaDeviceReset).  Those first calls must
// happen outside any stream capture; inside one they fail with
// cudaErrorStreamCaptureUnsupported instead of using a stale address.
// ---------------------------------------------------------------------------
constexpr int64_t kStaticEigElems = (int64_t)(8 << 20) / 16;
static __device__ __align__(256) double2 g_eig_scratch[kStaticEigElems];

namespace {

constexpr int kMaxDevices = 64;

// The array's device address, cached per device together with the identity
// of the CUDA context it was looked up in.  A device reset (cudaDeviceReset)
// destroys the primary context and the module with it; the next context may
// load the module at another address.  Context handles can be reused after a
// reset, context IDs (cuCtxGetId) are unique for the life of the process, so
// the cache is keyed by the ID.
struct ScratchAddr {
  unsigned long long ctx_id = 0;
  double2* addr = nullptr;
};
ScratchAddr g_eig_scratch_addr[kMaxDevices];
std::mutex g_eig_scratch_mutex;

typedef CUresult (*PfnCtxGetCurrent)(CUcontext*);
typedef CUresult (*PfnCtxGetId)(CUcontext, unsigned long long*);

// ID of the calling thread's current CUDA context (0 and an error if unknown)
cudaError_t current_ctx_id(unsigned long long* id) {
  static PfnCtxGetCurrent get_current = nullptr;
  static PfnCtxGetId get_id = nullptr;
  if (!get_current || !get_id) {
    void* f1 = nullptr;
    void* f2 = nullptr;
    cudaDriverEntryPointQueryResult q1, q2;
    cudaError_t e = cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000, cudaEnableDefault, &q1);
    if (e == cudaSuccess) e = cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2);
    if (e != cudaSuccess) return e;
    if (q1 != cudaDriverEntryPointSuccess || q2 != cudaDriverEntryPointSuccess || !f1 || !f2)
      return cudaErrorNotSupported;
    get_current = (PfnCtxGetCurrent)f1;
    get_id = (PfnCtxGetId)f2;
  }
  CUcontext ctx = nullptr;
  if (get_current(&ctx) != CUDA_SUCCESS || !ctx) return cudaErrorDeviceUninitialized;
  if (get_id(ctx, id) != CUDA_SUCCESS) return cudaErrorDeviceUninitialized;
  return cudaSuccess;
}

// U[b] = g_eig_scratch + b*d*d; matrix b of the batch is one block
__global__ void __launch_bounds__(kThreads) k_eig_strided(const double2* __restrict__ rho,
                                                          double2* __restrict__ rhoinv, double2* U,
                                                          int d, double eps) {
  const int64_t o = (int64_t)blockIdx.x * d * d;
  EigTask t;
  t.rho = rho + o;
  t.rhoinv = rhoinv + o;
  t.U = U + o;
  t.d = d;
  t.pad = 0;
  eig_body(t, eps);
}

}  // namespace

int64_t static_eig_capacity() { return kStaticEigElems; }

cudaError_t launch_rho_inverse_static(const double2* rho, double2* rhoinv, int n_mats, int d,
                                      double eps, cudaStream_t s) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
  double2* scratch = nullptr;
  {
    unsigned long long id = 0;
    e = current_ctx_id(&id);
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> lock(g_eig_scratch_mutex);
    ScratchAddr& cache = g_eig_scratch_addr[dev];
    if (!cache.addr || cache.ctx_id != id) {
      // set-up once per device and context, with that device current; it
      // may load the module, so it must not happen inside a stream capture
      cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
      e = cudaStreamIsCapturing(s, &cs);
      if (e != cudaSuccess) return e;
      if (cs != cudaStreamCaptureStatusNone) return cudaErrorStreamCaptureUnsupported;
      void* p = nullptr;
      e = cudaGetSymbolAddress(&p, g_eig_scratch);
      if (e != cudaSuccess) return e;
      cache.addr = (double2*)p;
      cache.ctx_id = id;
    }
    scratch = cache.addr;
  }
  const int64_t sm = eig_smem_bytes(d);
  e = cudaFuncSetAttribute(k_eig_strided, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  if (e != cudaSuccess) return e;
  k_eig_strided<<<(unsigned)n_mats, kThreads, sm, s>>>(rho, rhoinv, scratch, d, eps);
  return cudaGetLastError();
}


// ---------------------------------------------------------------------------
// Householder QR of node tensors (qrOrthogonal, complex128 on the FP64 pipe).
// One block per node: A (m x n, column-major: the node tensor as a
// (lastBefore x d_up) matrix) is factored in place by n reflectors
// H_j = I - tau_j v_j v_j^H (v_j in A[j:m, j], the diagonal of R aside);
// then the thin Q = H_0 ... H_{n-1} [I; 0] is formed in the scratch Qs and
// copied over A, and R (n x n, column-major, upper triangular) is written to R.
// Reflector j maps x = A[j:m, j] to alpha e_1 with alpha = -e^{i arg x_0} |x|
// (the LAPACK / Eigen choice).  Warps take columns (k = j + 1 + warp,
// j + 1 + warp + 8, ...), each column's dot product a warp reduction.
// ---------------------------------------------------------------------------
__device__ __forceinline__ double2 warp_sum2(double2 v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    v.x += __shfl_xor_sync(0xffffffffu, v.x, o);
    v.y += __shfl_xor_sync(0xffffffffu, v.y, o);
  }
  return v;
}

__global__ void __launch_bounds__(kThreads) k_house_qr(const QRTask* __restrict__ tasks) {
  const QRTask t = tasks[blockIdx.x];
  double2* __restrict__ A = t.A;
  const int m = t.m, n = t.n, steps = min(m, n);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31, nw = kThreads / 32;
  __shared__ double s_tau[112];
  __shared__ double2 s_alpha[112];
  __shared__ double s_nrm[kThreads / 32];
  for (int j = 0; j < steps; ++j) {
    double2* x = A + (int64_t)m * j;
    // |x|^2 over rows j..m-1
    double q = 0.0;
    for (int i = j + tid; i < m; i += kThreads) q += x[i].x * x[i].x + x[i].y * x[i].y;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) q += __shfl_xor_sync(0xffffffffu, q, o);
    if (lane == 0) s_nrm[warp] = q;
    __syncthreads();
    if (tid == 0) {
      double nrm2 = 0.0;
      for (int w = 0; w < nw; ++w) nrm2 += s_nrm[w];
      const double2 x0 = x[j];
      const double ax0 = sqrt(x0.x * x0.x + x0.y * x0.y), nrm = sqrt(nrm2);
      const double2 ph = ax0 > 0.0 ? make_double2(x0.x / ax0, x0.y / ax0) : make_double2(1.0, 0.0);
      const double2 alpha = make_double2(-ph.x * nrm, -ph.y * nrm);
      const double2 v0 = make_double2(x0.x - alpha.x, x0.y - alpha.y);
      const double vn2 = nrm2 - ax0 * ax0 + v0.x * v0.x + v0.y * v0.y;
      s_tau[j] = vn2 > 0.0 ? 2.0 / vn2 : 0.0;
      s_alpha[j] = nrm2 > 0.0 ? alpha : make_double2(0.0, 0.0);
      x[j] = v0;  // v_j = x - alpha e_1 (rows j..m-1 of column j)
    }
    __syncthreads();
    const double tau = s_tau[j];
    // columns k > j: a -= tau v (v^H a)
    for (int k = j + 1 + warp; k < n; k += nw) {
      double2* a = A + (int64_t)m * k;
      double2 w = make_double2(0.0, 0.0);
      for (int i = j + lane; i < m; i += 32) {
        const double2 vi = x[i], ai = a[i];
        w.x += vi.x * ai.x + vi.y * ai.y;  // conj(v) a
        w.y += vi.x * ai.y - vi.y * ai.x;
      }
      w = warp_sum2(w);
      const double2 tw = make_double2(tau * w.x, tau * w.y);
      for (int i = j + lane; i < m; i += 32) {
        const double2 vi = x[i];
        a[i].x -= vi.x * tw.x - vi.y * tw.y;
        a[i].y -= vi.x * tw.y + vi.y * tw.x;
      }
    }
    __syncthreads();
  }
  // R: the upper triangle above the diagonal is final in A, the diagonal is alpha
  for (int e = tid; e < n * n; e += kThreads) {
    const int i = e % n, k = e / n;
    double2 r = make_double2(0.0, 0.0);
    if (i < k && i < m) r = A[i + (int64_t)m * k];
    else if (i == k && i < steps) r = s_alpha[i];
    t.R[e] = r;
  }
  // thin Q = H_0 ... H_{n-1} [I; 0], accumulated backwards in Qs
  double2* __restrict__ Q = t.Qs;
  for (int64_t e = tid; e < (int64_t)m * n; e += kThreads) {
    const int i = (int)(e % m), k = (int)(e / m);
    Q[e] = make_double2(i == k ? 1.0 : 0.0, 0.0);
  }
  __syncthreads();
  for (int j = steps - 1; j >= 0; --j) {
    const double2* v = A + (int64_t)m * j;
    const double tau = s_tau[j];
    for (int k = j + warp; k < n; k += nw) {
      double2* qk = Q + (int64_t)m * k;
      double2 w = make_double2(0.0, 0.0);
      for (int i = j + lane; i < m; i += 32) {
        const double2 vi = v[i], ai = qk[i];
        w.x += vi.x * ai.x + vi.y * ai.y;
        w.y += vi.x * ai.y - vi.y * ai.x;
      }
      w = warp_sum2(w);
      const double2 tw = make_double2(tau * w.x, tau * w.y);
      for (int i = j + lane; i < m; i += 32) {
        const double2 vi = v[i];
        qk[i].x -= vi.x * tw.x - vi.y * tw.y;
        qk[i].y -= vi.x * tw.y + vi.y * tw.x;
      }
    }
    __syncthreads();
  }
  for (int64_t e = tid; e < (int64_t)m * n; e += kThreads) A[e] = Q[e];
}

cudaError_t launch_house_qr(const void* tasks, int n_tasks, cudaStream_t s) {
  if (n_tasks <= 0) return cudaSuccess;
  k_house_qr<<<(unsigned)n_tasks, kThreads, 0, s>>>(static_cast<const QRTask*>(tasks));
  return cudaGetLastError();
}

}  // namespace qt
