// qt_oracle.cpp -- CPU FP64 restatement of QuTree's H.Psi sweep.
//
// TEST INFRASTRUCTURE ONLY.  This file is the checker the GPU library is
// compared against and the CPU baseline timed beside it.  Nothing in the
// product (qutree_gb300/, include/) links, loads or calls it.
//
// It restates, in plain C++ over complex<double>, the reference algorithm of
// QuTree's Derivative() (src/TreeClasses/HamiltonianRepresentation.cpp:6-81)
// with the same call sequence and, for the loop kernels, the same summation
// order as the Fortran kernels the reference calls:
//   matvec   src/Core/LA_lib.f:34-81     (mode product, square matrix)
//   rhomat   src/Core/LA_lib.f:718-762   (hole product, square)
//   matrixTensor1 / contraction1         include/Core/Tensor_Implementation.h:463-551
//   matrixTensor2 / contraction2 (zgemm) src/Core/TensorBLAS.cpp:124-225
// Two primitive back ends are selectable per call: LOOPS (the Fortran/loop
// kernels) and BLAS (the TensorBLAS path: zgemm per slice + transpose, or
// transposeBC + zgemm^H), the latter through a caller-supplied cblas_zgemm.
//
// Inputs are the flat descriptors of include/qtgpu.h (tree, operator table,
// SOP, wavefunction), so the oracle and the GPU library read identical data.
#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstring>
#include <functional>
#include <map>
#include <set>
#include <vector>

using cd = std::complex<double>;

namespace {

// ---------------------------------------------------------------------------
// zgemm back end for the BLAS primitives
// ---------------------------------------------------------------------------
// cblas_zgemm(order, transA, transB, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc)
typedef void (*zgemm_lp64_t)(int, int, int, int, int, int, const void*, const void*, int,
                             const void*, int, const void*, void*, int);
typedef void (*zgemm_ilp64_t)(int, int, int, int64_t, int64_t, int64_t, const void*, const void*,
                              int64_t, const void*, int64_t, const void*, void*, int64_t);
void* g_zgemm = nullptr;
int g_zgemm_ilp64 = 0;
enum { kColMajor = 102, kNoTrans = 111, kTrans = 112, kConjTrans = 113 };

// Column-major C = alpha op(A) op(B) + beta C, with a naive fallback.
void zgemm(int ta, int tb, int64_t m, int64_t n, int64_t k, cd alpha, const cd* A, int64_t lda,
           const cd* B, int64_t ldb, cd beta, cd* C, int64_t ldc) {
  if (g_zgemm) {
    if (g_zgemm_ilp64)
      ((zgemm_ilp64_t)g_zgemm)(kColMajor, ta, tb, m, n, k, &alpha, A, lda, B, ldb, &beta, C, ldc);
    else
      ((zgemm_lp64_t)g_zgemm)(kColMajor, ta, tb, (int)m, (int)n, (int)k, &alpha, A, (int)lda, B,
                              (int)ldb, &beta, C, (int)ldc);
    return;
  }
  for (int64_t j = 0; j < n; ++j)
    for (int64_t i = 0; i < m; ++i) {
      cd s = 0;
      for (int64_t l = 0; l < k; ++l) {
        cd a = (ta == kNoTrans) ? A[i + l * lda] : A[l + i * lda];
        if (ta == kConjTrans) a = std::conj(a);
        cd b = (tb == kNoTrans) ? B[l + j * ldb] : B[j + l * ldb];
        if (tb == kConjTrans) b = std::conj(b);
        s += a * b;
      }
      C[i + j * ldc] = alpha * s + (beta == cd(0) ? cd(0) : beta * C[i + j * ldc]);
    }
}

// ---------------------------------------------------------------------------
// Primitive kernels
// ---------------------------------------------------------------------------
enum Backend { LOOPS = 0, BLAS = 1 };

// LA_lib.f matvec: mulpsi(i,k,j) += matrix(k,l) * psi(i,l,j), loops j,k,l,i.
void matvec(cd* C, const cd* B, const cd* h, int64_t a, int64_t b, int64_t c, bool add) {
  if (!add) std::memset((void*)C, 0, sizeof(cd) * a * b * c);
  for (int64_t j = 0; j < c; ++j)
    for (int64_t k = 0; k < a; ++k)
      for (int64_t l = 0; l < a; ++l) {
        const cd m = h[k + l * a];
        const cd* bp = B + (l + j * a) * b;
        cd* cp = C + (k + j * a) * b;
        for (int64_t i = 0; i < b; ++i) cp[i] += m * bp[i];
      }
}

// matrixTensor1 (include/Core/Tensor_Implementation.h:533-551), rectangular h (activeC x activeB).
void matrixTensor1(cd* C, const cd* h, const cd* B, int64_t before, int64_t activeB,
                   int64_t activeC, int64_t after, bool zero) {
  if (zero) std::memset((void*)C, 0, sizeof(cd) * before * activeC * after);
  for (int64_t aft = 0; aft < after; ++aft)
    for (int64_t act = 0; act < activeB; ++act)
      for (int64_t actC = 0; actC < activeC; ++actC) {
        const cd m = h[act * activeC + actC];
        for (int64_t bef = 0; bef < before; ++bef)
          C[activeC * before * aft + actC * before + bef] +=
              m * B[activeB * before * aft + act * before + bef];
      }
}

// LA_lib.f rhomat: matrix(j,i) = sum conjg(bra(n,j,m)) * ket(n,i,m) (always overwrites).
void rhomat(cd* S, const cd* bra, const cd* ket, int64_t a, int64_t b, int64_t c) {
  for (int64_t x = 0; x < a * a; ++x) S[x] = 0;
  if (b != 1) {
    for (int64_t m = 0; m < c; ++m)
      for (int64_t i = 0; i < a; ++i)
        for (int64_t j = 0; j < a; ++j) {
          cd s = S[j + i * a];
          const cd* bp = bra + (j + m * a) * b;
          const cd* kp = ket + (i + m * a) * b;
          for (int64_t n = 0; n < b; ++n) s += std::conj(bp[n]) * kp[n];
          S[j + i * a] = s;
        }
  } else if (c > a) {
    for (int64_t i = 0; i < a; ++i)
      for (int64_t j = 0; j < a; ++j)
        for (int64_t m = 0; m < c; ++m) S[j + i * a] += std::conj(bra[j + m * a]) * ket[i + m * a];
  } else {
    for (int64_t m = 0; m < c; ++m)
      for (int64_t i = 0; i < a; ++i)
        for (int64_t j = 0; j < a; ++j) S[j + i * a] += std::conj(bra[j + m * a]) * ket[i + m * a];
  }
}

// contraction1 (include/Core/Tensor_Implementation.h:463-479): h(b,b2) += conj(bra(a,b,c)) ket(a,b2,c).
void contraction1(cd* h, const cd* bra, const cd* ket, int64_t A, int64_t B, int64_t B2, int64_t C,
                  bool zero) {
  if (zero) std::memset((void*)h, 0, sizeof(cd) * B * B2);
  for (int64_t a = 0; a < A; ++a)
    for (int64_t b = 0; b < B; ++b)
      for (int64_t b2 = 0; b2 < B2; ++b2)
        for (int64_t c = 0; c < C; ++c)
          h[b + b2 * B] += std::conj(bra[a + b * A + c * A * B]) * ket[a + b2 * A + c * A * B2];
}

// transpose (src/Core/TensorBLAS.cpp:13-34): dest[dim2, dim1] = src[dim1, dim2] + beta*dest.
void transpose(cd* dest, const cd* src, int64_t dim1, int64_t dim2, cd beta) {
  const int64_t stride = 12;
  for (int64_t jj = 0; jj < dim1; jj += stride) {
    const int64_t jend = std::min(dim1, jj + stride);
    for (int64_t ii = 0; ii < dim2; ii += stride) {
      const int64_t iend = std::min(dim2, ii + stride);
      for (int64_t i = ii; i < iend; ++i)
        for (int64_t j = jj; j < jend; ++j)
          dest[i + dim2 * j] = src[j + dim1 * i] + beta * dest[i + dim2 * j];
    }
  }
}

// transposeBC (src/Core/TensorBLAS.cpp:91-102): dest[a, c, b] = src[a, b, c].
void transposeBC(cd* dest, const cd* src, int64_t A, int64_t B, int64_t C) {
  for (int64_t c = 0; c < C; ++c)
    for (int64_t b = 0; b < B; ++b)
      std::memcpy((void*)(dest + c * A + b * A * C), src + b * A + c * A * B, A * sizeof(cd));
}

std::vector<cd> g_work1, g_work2;

// Mode-k product C = h x_k B with (before, activeB, after) geometry.
//   LOOPS: matrixTensor (include/Core/Tensor_Implementation.h:553-577): square -> matvec.
//   BLAS : matrixTensor2 (src/Core/TensorBLAS.cpp:124-173): zgemm per after slice + transpose.
void mode_product(Backend be, cd* C, const cd* h, const cd* B, int64_t before, int64_t activeB,
                  int64_t activeC, int64_t after, bool zero) {
  if (be == LOOPS) {
    if (activeB == activeC)
      matvec(C, B, h, activeB, before, after, !zero);
    else
      matrixTensor1(C, h, B, before, activeB, activeC, after, zero);
    return;
  }
  const cd z(1.0), zz(zero ? 0.0 : 1.0);
  if (before == 1) {
    zgemm(kNoTrans, kNoTrans, activeC, after, activeB, z, h, activeC, B, activeB, zz, C, activeC);
    return;
  }
  const int64_t pref = before * activeB, prefC = before * activeC;
  if ((int64_t)g_work1.size() < prefC * after) g_work1.resize(prefC * after);
  cd* D = g_work1.data();
  for (int64_t aft = 0; aft < after; ++aft) {
    zgemm(kNoTrans, kTrans, activeC, before, activeB, z, h, activeC, B + aft * pref, before,
          cd(0.0), D + aft * prefC, activeC);
    transpose(C + aft * prefC, D + aft * prefC, activeC, before, zz);
  }
}

// Hole product S(a,a') = sum conj(A[b,a,c]) B[b,a',c].
//   LOOPS: contraction (include/Core/Tensor_Implementation.h:481-531): square -> rhomat.
//   BLAS : contraction2 (src/Core/TensorBLAS.cpp:200-225): transposeBC both + zgemm(C,N).
void hole_product(Backend be, cd* S, const cd* A, const cd* B, int64_t before, int64_t activeA,
                  int64_t activeB, int64_t after) {
  if (be == LOOPS) {
    if (activeA == activeB)
      rhomat(S, A, B, activeA, before, after);
    else
      contraction1(S, A, B, before, activeA, activeB, after, true);
    return;
  }
  const int64_t AC = before * after;
  if ((int64_t)g_work1.size() < AC * activeA) g_work1.resize(AC * activeA);
  if ((int64_t)g_work2.size() < AC * activeB) g_work2.resize(AC * activeB);
  transposeBC(g_work1.data(), A, before, activeA, after);
  transposeBC(g_work2.data(), B, before, activeB, after);
  zgemm(kConjTrans, kNoTrans, activeA, activeB, AC, cd(1.0), g_work1.data(), AC, g_work2.data(),
        AC, cd(0.0), S, activeA);
}

// ---------------------------------------------------------------------------
// Small dense linear algebra (the reference calls Eigen here)
// ---------------------------------------------------------------------------
// Hermitian eigendecomposition by cyclic complex Jacobi rotations; eigenvalues
// ascending, eigenvectors as columns with QuTree's phase convention
// (Re U(0,i) >= 0, include/Core/Matrix_Implementation.h:284-309).
void herm_eig(int n, const cd* A, cd* U, double* w) {
  std::vector<cd> a(A, A + n * n);
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) U[i + j * n] = (i == j) ? 1.0 : 0.0;
  // symmetrise (take the Hermitian part)
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < i; ++j) {
      cd v = 0.5 * (a[i + j * n] + std::conj(a[j + i * n]));
      a[i + j * n] = v;
      a[j + i * n] = std::conj(v);
    }
  for (int i = 0; i < n; ++i) a[i + i * n] = a[i + i * n].real();
  for (int sweep = 0; sweep < 100; ++sweep) {
    double off = 0, diag = 0;
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i) {
        if (i != j) off += std::norm(a[i + j * n]);
        else diag += std::norm(a[i + j * n]);
      }
    if (off <= 1e-30 * (diag + 1e-300) || off == 0.0) break;
    for (int p = 0; p < n - 1; ++p)
      for (int q = p + 1; q < n; ++q) {
        cd apq = a[p + q * n];
        double ab = std::abs(apq);
        if (ab == 0.0) continue;
        double app = a[p + p * n].real(), aqq = a[q + q * n].real();
        // rotation annihilating a(p,q): phase e = apq/|apq|
        cd e = apq / ab;
        double theta = 0.5 * std::atan2(2.0 * ab, aqq - app);
        double c = std::cos(theta), s = std::sin(theta);
        // columns p,q of a: a' = a * G, G = [[c, s*e],[-s*conj(e), c]]
        for (int k = 0; k < n; ++k) {
          cd akp = a[k + p * n], akq = a[k + q * n];
          a[k + p * n] = c * akp - s * std::conj(e) * akq;
          a[k + q * n] = s * e * akp + c * akq;
        }
        for (int k = 0; k < n; ++k) {
          cd apk = a[p + k * n], aqk = a[q + k * n];
          a[p + k * n] = c * apk - s * e * aqk;
          a[q + k * n] = s * std::conj(e) * apk + c * aqk;
        }
        for (int k = 0; k < n; ++k) {
          cd ukp = U[k + p * n], ukq = U[k + q * n];
          U[k + p * n] = c * ukp - s * std::conj(e) * ukq;
          U[k + q * n] = s * e * ukp + c * ukq;
        }
        a[p + q * n] = 0;
        a[q + p * n] = 0;
      }
  }
  std::vector<int> idx(n);
  for (int i = 0; i < n; ++i) idx[i] = i;
  std::vector<double> d(n);
  for (int i = 0; i < n; ++i) d[i] = a[i + i * n].real();
  std::stable_sort(idx.begin(), idx.end(), [&](int x, int y) { return d[x] < d[y]; });
  std::vector<cd> Us(U, U + n * n);
  for (int j = 0; j < n; ++j) {
    w[j] = d[idx[j]];
    double sgn = (Us[0 + idx[j] * n].real() < 0) ? -1.0 : 1.0;
    for (int i = 0; i < n; ++i) U[i + j * n] = sgn * Us[i + idx[j] * n];
  }
}

// Gauss-Jordan inverse with partial pivoting (stands in for Eigen's inverse(),
// Matrix::cInv, include/Core/Matrix_Implementation.h:311-329).
void inverse(int n, const cd* A, cd* X) {
  std::vector<cd> a(A, A + n * n);
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) X[i + j * n] = (i == j) ? 1.0 : 0.0;
  for (int col = 0; col < n; ++col) {
    int piv = col;
    double best = std::abs(a[col + col * n]);
    for (int r = col + 1; r < n; ++r)
      if (std::abs(a[r + col * n]) > best) best = std::abs(a[r + col * n]), piv = r;
    if (piv != col)
      for (int j = 0; j < n; ++j) {
        std::swap(a[col + j * n], a[piv + j * n]);
        std::swap(X[col + j * n], X[piv + j * n]);
      }
    cd d = 1.0 / a[col + col * n];
    for (int j = 0; j < n; ++j) a[col + j * n] *= d, X[col + j * n] *= d;
    for (int r = 0; r < n; ++r) {
      if (r == col) continue;
      cd f = a[r + col * n];
      if (f == cd(0)) continue;
      for (int j = 0; j < n; ++j) {
        a[r + j * n] -= f * a[col + j * n];
        X[r + j * n] -= f * X[col + j * n];
      }
    }
  }
}

// ---------------------------------------------------------------------------
// Tree / operator / SOP descriptors
// ---------------------------------------------------------------------------
struct Tree {
  int n = 0;
  std::vector<std::vector<int>> shape;
  std::vector<int> parent, child_idx, leaf_mode;
  std::vector<std::vector<int>> children;
  std::vector<int64_t> off, size;
  std::map<int, int> leaf_node;
  int64_t before(int node, int k) const {
    int64_t b = 1;
    for (int i = 0; i < k; ++i) b *= shape[node][i];
    return b;
  }
  int64_t after(int node, int k) const {
    int64_t a = 1;
    for (size_t i = k + 1; i < shape[node].size(); ++i) a *= shape[node][i];
    return a;
  }
  int last(int node) const { return (int)shape[node].size() - 1; }
  int dup(int node) const { return shape[node].back(); }
  bool top(int node) const { return parent[node] < 0; }
  bool bottom(int node) const { return leaf_mode[node] >= 0; }
};

Tree make_tree(int n_nodes, const int* order, const int* dims, const int* parent,
               const int* child_idx, const int* leaf_mode) {
  Tree t;
  t.n = n_nodes;
  t.shape.resize(n_nodes);
  t.children.resize(n_nodes);
  t.off.resize(n_nodes + 1);
  t.size.resize(n_nodes);
  int p = 0;
  t.off[0] = 0;
  for (int i = 0; i < n_nodes; ++i) {
    int64_t s = 1;
    for (int k = 0; k < order[i]; ++k) {
      t.shape[i].push_back(dims[p + k]);
      s *= dims[p + k];
    }
    p += order[i];
    t.size[i] = s;
    t.off[i + 1] = t.off[i] + s;
    t.parent.push_back(parent[i]);
    t.child_idx.push_back(child_idx[i]);
    t.leaf_mode.push_back(leaf_mode[i]);
    if (leaf_mode[i] >= 0) t.leaf_node[leaf_mode[i]] = i;
  }
  for (int i = 0; i < n_nodes; ++i)
    if (parent[i] >= 0) {
      auto& ch = t.children[parent[i]];
      if ((int)ch.size() <= child_idx[i]) ch.resize(child_idx[i] + 1, -1);
      ch[child_idx[i]] = i;
    }
  return t;
}

struct Ops {
  const int* kind;
  const int* dim;
  const int64_t* off;
  const cd* data;
};

struct Sop {
  int n_terms;
  const cd* coeff;
  const int* ptr;
  const int* mode;
  const int* op;
};

// Active nodes of a term: the union of the leaf-to-root paths of its target
// leaves (SparseTree::SparseInitialize with tail = true,
// src/TreeClasses/SparseTree.cpp:33-89), in ascending address order.
std::vector<char> active_nodes(const Tree& t, const Sop& s, int l) {
  std::vector<char> act(t.n, 0);
  for (int f = s.ptr[l]; f < s.ptr[l + 1]; ++f) {
    int node = t.leaf_node.at(s.mode[f]);
    while (node >= 0) {
      act[node] = 1;
      node = t.parent[node];
    }
  }
  return act;
}

// Apply one leaf operator to a bottom tensor (p, d_up): dense -> mode-0
// product; diagonal -> elementwise (DVRBasis::applyX/X2,
// src/TreeShape/LeafTypes/DVRBasis.cpp:8-58; LeafMatrix::apply,
// src/TreeOperators/LeafMatrix.cpp:37-40).
void apply_leaf_op(Backend be, const Ops& ops, int op, cd* out, const cd* in, int p, int dup) {
  const cd* d = ops.data + ops.off[op];
  if (ops.kind[op] == 0) {
    mode_product(be, out, d, in, 1, p, p, dup, true);
  } else {
    for (int n = 0; n < dup; ++n)
      for (int i = 0; i < p; ++i) out[i + n * p] = d[i] * in[i + n * p];
  }
}

// MLO::apply(Phi, leaf) (src/TreeOperators/MultiLeafOperator.cpp:11-37):
// every factor of the term that targets this leaf, in list order.
void apply_mlo(Backend be, const Ops& ops, const Sop& s, int l, int mode, cd* buf, cd* tmp,
               int p, int dup) {
  for (int f = s.ptr[l]; f < s.ptr[l + 1]; ++f) {
    if (s.mode[f] != mode) continue;
    apply_leaf_op(be, ops, s.op[f], tmp, buf, p, dup);
    std::memcpy((void*)buf, tmp, sizeof(cd) * p * dup);
  }
}

struct Sweep {
  const Tree& t;
  const Ops& ops;
  const Sop& s;
  Backend be;
  const cd* psi;  // current wavefunction (the integrator re-points it)
  std::vector<std::vector<char>> act;          // [term][node]
  std::vector<std::vector<int64_t>> moff;      // sparse matrix offsets [term][node]
  std::vector<cd> hmat, hcon;                  // sparse matrix trees
  std::vector<int64_t> roff;                   // per-node matrix offsets
  std::vector<cd> rho, rhoinv;
  double eps;

  Sweep(const Tree& t_, const Ops& o_, const Sop& s_, Backend be_, const cd* psi_, double eps_)
      : t(t_), ops(o_), s(s_), be(be_), psi(psi_), eps(eps_) {
    int64_t acc = 0;
    act.resize(s.n_terms);
    moff.resize(s.n_terms);
    for (int l = 0; l < s.n_terms; ++l) {
      act[l] = active_nodes(t, s, l);
      moff[l].assign(t.n, -1);
      for (int n = 0; n < t.n; ++n)
        if (act[l][n]) {
          moff[l][n] = acc;
          acc += (int64_t)t.dup(n) * t.dup(n);
        }
    }
    hmat.assign(acc, 0);
    hcon.assign(acc, 0);
    roff.resize(t.n + 1);
    roff[0] = 0;
    for (int n = 0; n < t.n; ++n) roff[n + 1] = roff[n] + (int64_t)t.dup(n) * t.dup(n);
    rho.assign(roff[t.n], 0);
    rhoinv.assign(roff[t.n], 0);
  }

  const cd* phi(int n) const { return psi + t.off[n]; }
  int64_t N(int n) const { return t.size[n]; }

  // C = h x_k B on node geometry (square h of the mode's dim)
  void mp(cd* C, const cd* h, const cd* B, int node, int k) {
    int a = t.shape[node][k];
    mode_product(be, C, h, B, t.before(node, k), a, a, t.after(node, k), true);
  }
  void hp(cd* S, const cd* A, const cd* B, int node, int k) {
    int a = t.shape[node][k];
    hole_product(be, S, A, B, t.before(node, k), a, a, t.after(node, k));
  }

  // ---- density matrices: TreeFunctions::contraction(Rho, Psi, tree, true)
  // (include/TreeClasses/MatrixTreeFunctions_Implementation.h:59-103)
  void density() {
    std::vector<cd> K;
    for (int n = t.n - 1; n >= 0; --n) {
      if (t.top(n)) {
        int d = t.dup(n);
        for (int i = 0; i < d; ++i) rho[roff[n] + i + i * d] = 1.0;
        continue;
      }
      int p = t.parent[n];
      K.assign(N(p), 0);
      mp(K.data(), &rho[roff[p]], phi(p), p, t.last(p));
      hp(&rho[roff[n]], phi(p), K.data(), p, t.child_idx[n]);
    }
  }

  // ---- spectral decomposition and regularised inverse
  // (src/TreeClasses/SpectralDecompositionTree.cpp:30-48;
  //  include/Core/Vector_Implementation.h:266-280; toMatrix :636-649)
  void invert() {
    for (int n = 0; n < t.n; ++n) {
      int d = t.dup(n);
      std::vector<cd> U(d * d);
      std::vector<double> w(d);
      herm_eig(d, &rho[roff[n]], U.data(), w.data());
      for (int i = 0; i < d; ++i) w[i] = 1.0 / (w[i] + eps * std::exp(-w[i] / eps));
      cd* R = &rhoinv[roff[n]];
      for (int i = 0; i < d; ++i)
        for (int j = 0; j < d; ++j) {
          cd acc = 0;
          for (int k = 0; k < d; ++k) acc += U[i + k * d] * w[k] * std::conj(U[j + k * d]);
          R[i + j * d] = acc;
        }
    }
  }

  // ---- represent (include/TreeClasses/SparseMatrixTreeFunctions_Implementation.h:17-78)
  void represent() {
    std::vector<cd> A, B;
    for (int l = 0; l < s.n_terms; ++l)
      for (int n = 0; n < t.n; ++n) {
        if (!act[l][n] || t.top(n)) continue;
        A.assign(phi(n), phi(n) + N(n));
        B.assign(N(n), 0);
        if (t.bottom(n)) {
          apply_mlo(be, ops, s, l, t.leaf_mode[n], A.data(), B.data(), t.shape[n][0], t.dup(n));
        } else {
          for (size_t k = 0; k < t.children[n].size(); ++k) {
            int c = t.children[n][k];
            if (!act[l][c]) continue;
            mp(B.data(), &hmat[moff[l][c]], A.data(), n, (int)k);
            std::swap(A, B);
          }
        }
        hp(&hmat[moff[l][n]], phi(n), A.data(), n, t.last(n));
      }
  }

  // ---- mean fields (include/TreeClasses/SparseMatrixTreeFunctions_Implementation.h:144-203,298-351)
  void meanfield() {
    std::vector<cd> A, B;
    for (int l = 0; l < s.n_terms; ++l)
      for (int n = t.n - 1; n >= 0; --n) {
        if (!act[l][n]) continue;
        if (t.top(n)) {
          int d = t.dup(n);
          for (int i = 0; i < d; ++i) hcon[moff[l][n] + i + i * d] = 1.0;
          continue;
        }
        int p = t.parent[n];
        A.assign(phi(p), phi(p) + N(p));
        B.assign(N(p), 0);
        for (size_t k = 0; k < t.children[p].size(); ++k) {
          int c = t.children[p][k];
          if ((int)k == t.child_idx[n] || !act[l][c]) continue;
          mp(B.data(), &hmat[moff[l][c]], A.data(), p, (int)k);
          std::swap(A, B);
        }
        if (!t.top(p)) {
          mp(B.data(), &hcon[moff[l][p]], A.data(), p, t.last(p));
          std::swap(A, B);
        }
        hp(&hcon[moff[l][n]], phi(p), A.data(), p, t.child_idx[n]);
      }
  }

  // ---- Apply (src/TreeClasses/HamiltonianRepresentation.cpp:6-43)
  void apply(int n, cd* dPhi) {
    std::vector<cd> A, B;
    std::fill(dPhi, dPhi + N(n), cd(0));
    for (int l = 0; l < s.n_terms; ++l) {
      if (!act[l][n]) continue;
      A.resize(N(n));
      B.assign(N(n), 0);
      for (int64_t i = 0; i < N(n); ++i) A[i] = s.coeff[l] * phi(n)[i];
      if (t.bottom(n)) {
        apply_mlo(be, ops, s, l, t.leaf_mode[n], A.data(), B.data(), t.shape[n][0], t.dup(n));
      } else {
        for (size_t k = 0; k < t.children[n].size(); ++k) {
          int c = t.children[n][k];
          if (!act[l][c]) continue;
          mp(B.data(), &hmat[moff[l][c]], A.data(), n, (int)k);
          std::swap(A, B);
        }
      }
      if (!t.top(n)) {
        // multStateAB(dPhi, hhole[node], Psi, false)
        int d = t.dup(n);
        mode_product(be, dPhi, &hcon[moff[l][n]], A.data(), N(n) / d, d, d, 1, false);
      } else {
        for (int64_t i = 0; i < N(n); ++i) dPhi[i] += A[i];
      }
    }
  }

  // ---- LayerDerivative (src/TreeClasses/HamiltonianRepresentation.cpp:53-72)
  void layer_derivative(int n, cd* dPhi, cd phase) {
    apply(n, dPhi);
    if (!t.top(n)) {
      int d = t.dup(n);
      int64_t R = N(n) / d;
      // projectOut (include/Core/Tensor_Implementation.h:873-910)
      std::vector<cd> S(d * d), Sinv(d * d), D(d * d), P(d * d), proj(N(n), 0);
      hp(S.data(), phi(n), phi(n), n, t.last(n));
      inverse(d, S.data(), Sinv.data());
      hp(D.data(), phi(n), dPhi, n, t.last(n));
      for (int i = 0; i < d; ++i)
        for (int j = 0; j < d; ++j) {
          cd acc = 0;
          for (int k = 0; k < d; ++k) acc += Sinv[i + k * d] * D[k + j * d];
          P[i + j * d] = acc;
        }
      // multStateArTB: C(i, m) += P(n, m) * B(i, n)
      for (int nn = 0; nn < d; ++nn)
        for (int m = 0; m < d; ++m) {
          cd pm = P[nn + m * d];
          const cd* bp = phi(n) + nn * R;
          cd* cp = proj.data() + m * R;
          for (int64_t i = 0; i < R; ++i) cp[i] += pm * bp[i];
        }
      for (int64_t i = 0; i < N(n); ++i) dPhi[i] -= proj[i];
      // multStateAB(rhoinv, dPhi)
      std::vector<cd> tmp(N(n));
      mode_product(be, tmp.data(), &rhoinv[roff[n]], dPhi, R, d, d, 1, true);
      std::copy(tmp.begin(), tmp.end(), dPhi);
    }
    cd f = -phase * cd(0.0, 1.0);
    for (int64_t i = 0; i < N(n); ++i) dPhi[i] *= f;
  }
};

}  // namespace

extern "C" {

int orc_version() { return 1; }

void orc_set_zgemm(void* fn, int ilp64) {
  g_zgemm = fn;
  g_zgemm_ilp64 = ilp64;
}

// Mode product C = h x_k B on a tensor of geometry (before, activeB, after);
// h is activeC x activeB column-major.  add != 0 accumulates into C.
void orc_mode_product(int backend, double* C, const double* h, const double* B, int64_t before,
                      int64_t activeB, int64_t activeC, int64_t after, int add) {
  mode_product((Backend)backend, (cd*)C, (const cd*)h, (const cd*)B, before, activeB, activeC,
               after, add == 0);
}

// Hole product S(a,a') = sum conj(A[b,a,c]) B[b,a',c].
void orc_hole_product(int backend, double* S, const double* A, const double* B, int64_t before,
                      int64_t activeA, int64_t activeB, int64_t after) {
  hole_product((Backend)backend, (cd*)S, (const cd*)A, (const cd*)B, before, activeA, activeB,
               after);
}

void orc_herm_eig(int n, const double* A, double* U, double* w) {
  herm_eig(n, (const cd*)A, (cd*)U, w);
}

void orc_inverse(int n, const double* A, double* X) { inverse(n, (const cd*)A, (cd*)X); }

// Size (complex elements) of the sparse matrix tree layout: for each term, for
// each active node in address order, a d_up x d_up matrix.
int64_t orc_sparse_size(int n_nodes, const int* order, const int* dims, const int* parent,
                        const int* child_idx, const int* leaf_mode, int n_terms,
                        const int* term_ptr, const int* term_mode) {
  Tree t = make_tree(n_nodes, order, dims, parent, child_idx, leaf_mode);
  Sop s{n_terms, nullptr, term_ptr, term_mode, nullptr};
  int64_t acc = 0;
  for (int l = 0; l < n_terms; ++l) {
    auto a = active_nodes(t, s, l);
    for (int n = 0; n < t.n; ++n)
      if (a[n]) acc += (int64_t)t.dup(n) * t.dup(n);
  }
  return acc;
}

// One full sweep: HamiltonianRepresentation::build + LayerDerivative at every
// node + Expectation.  Outputs (any may be null):
//   dpsi   : derivative, same layout as psi
//   rho, rhoinv : per-node d_up x d_up, nodes back to back
//   hmat, hcon  : sparse matrix trees (layout of orc_sparse_size)
//   energy : [Re h00, Im h00, Re S00, Im S00] with h00 = <Phi_top|H Phi_top>,
//            S00 = <Phi_top|Phi_top>
// Returns 0.
int orc_derivative(int backend, int n_nodes, const int* order, const int* dims, const int* parent,
                   const int* child_idx, const int* leaf_mode, int n_ops, const int* op_kind,
                   const int* op_dim, const int64_t* op_off, const double* op_data, int n_terms,
                   const double* coeff, const int* term_ptr, const int* term_mode,
                   const int* term_op, const double* psi, double eps, double phase_re,
                   double phase_im, double* dpsi, double* rho, double* rhoinv, double* hmat,
                   double* hcon, double* energy) {
  (void)n_ops;
  Tree t = make_tree(n_nodes, order, dims, parent, child_idx, leaf_mode);
  Ops ops{op_kind, op_dim, op_off, (const cd*)op_data};
  Sop s{n_terms, (const cd*)coeff, term_ptr, term_mode, term_op};
  Sweep sw(t, ops, s, (Backend)backend, (const cd*)psi, eps);
  sw.density();
  sw.invert();
  sw.represent();
  sw.meanfield();
  std::vector<cd> d(t.off[t.n]);
  cd phase(phase_re, phase_im);
  for (int n = 0; n < t.n; ++n) sw.layer_derivative(n, d.data() + t.off[n], phase);
  if (dpsi) std::memcpy(dpsi, d.data(), sizeof(cd) * d.size());
  if (rho) std::memcpy(rho, sw.rho.data(), sizeof(cd) * sw.rho.size());
  if (rhoinv) std::memcpy(rhoinv, sw.rhoinv.data(), sizeof(cd) * sw.rhoinv.size());
  if (hmat) std::memcpy(hmat, sw.hmat.data(), sizeof(cd) * sw.hmat.size());
  if (hcon) std::memcpy(hcon, sw.hcon.data(), sizeof(cd) * sw.hcon.size());
  if (energy) {
    // Expectation (src/TreeClasses/HamiltonianRepresentation.cpp:45-51)
    int top = t.n - 1;
    std::vector<cd> hphi(t.size[top]);
    sw.apply(top, hphi.data());
    int dt = t.dup(top);
    std::vector<cd> h(dt * dt), S(dt * dt);
    sw.hp(h.data(), sw.phi(top), hphi.data(), top, t.last(top));
    sw.hp(S.data(), sw.phi(top), sw.phi(top), top, t.last(top));
    energy[0] = h[0].real();
    energy[1] = h[0].imag();
    energy[2] = S[0].real();
    energy[3] = S[0].imag();
  }
  return 0;
}

// Fixed-step second-order constant-mean-field propagation with RK4 substeps
// (the scheme of CMFIntegrator::Integrate, src/Applications/CMFIntegrator.cpp:
// 25-174, without step-size control or re-orthonormalisation): per step,
// build at t; Psi_h = Psi(t) propagated to t+dt/2 with frozen matrices
// (n_sub RK4 steps); build at Psi_h; Psi(t) propagated to t+dt (2*n_sub RK4
// steps) with those matrices.  psi is updated in place.
int orc_cmf(int backend, int n_nodes, const int* order, const int* dims, const int* parent,
            const int* child_idx, const int* leaf_mode, int n_ops, const int* op_kind,
            const int* op_dim, const int64_t* op_off, const double* op_data, int n_terms,
            const double* coeff, const int* term_ptr, const int* term_mode, const int* term_op,
            double* psi_io, double eps, double phase_re, double phase_im, double dt, int n_steps,
            int n_sub) {
  (void)n_ops;
  Tree t = make_tree(n_nodes, order, dims, parent, child_idx, leaf_mode);
  Ops ops{op_kind, op_dim, op_off, (const cd*)op_data};
  Sop s{n_terms, (const cd*)coeff, term_ptr, term_mode, term_op};
  const int64_t N = t.off[t.n];
  cd* psi = (cd*)psi_io;
  cd phase(phase_re, phase_im);
  std::vector<cd> y0(N), y(N), in(N), k(N), acc(N);
  Sweep sw(t, ops, s, (Backend)backend, psi, eps);
  auto build = [&](const cd* at) {
    sw.psi = at;
    sw.density();
    sw.invert();
    sw.represent();
    sw.meanfield();
  };
  auto deriv = [&](const cd* at, cd* out) {
    sw.psi = at;
    for (int n = 0; n < t.n; ++n) sw.layer_derivative(n, out + t.off[n], phase);
  };
  auto rk4 = [&](std::vector<cd>& Y, double h, int steps) {
    for (int st = 0; st < steps; ++st) {
      const double w[4] = {1.0, 2.0, 2.0, 1.0};
      const double a[4] = {0.5 * h, 0.5 * h, h, 0.0};
      in = Y;
      for (int q = 0; q < 4; ++q) {
        deriv(in.data(), k.data());
        for (int64_t i = 0; i < N; ++i) acc[i] = (q == 0 ? cd(0) : acc[i]) + w[q] * k[i];
        if (q < 3)
          for (int64_t i = 0; i < N; ++i) in[i] = Y[i] + a[q] * k[i];
      }
      for (int64_t i = 0; i < N; ++i) Y[i] += (h / 6.0) * acc[i];
    }
  };
  for (int step = 0; step < n_steps; ++step) {
    y0.assign(psi, psi + N);
    build(y0.data());
    y = y0;
    rk4(y, 0.5 * dt / n_sub, n_sub);
    std::vector<cd> yh = y;
    build(yh.data());
    y = y0;
    rk4(y, 0.5 * dt / n_sub, 2 * n_sub);
    std::copy(y.begin(), y.end(), psi);
  }
  return 0;
}

// Frozen-matrix session (the LayerInterface of CMFIntegrator,
// src/Applications/CMFIntegrator.cpp:11-23, include/TreeClasses/LayerInterface.h):
// orc_frozen_build = HamiltonianRepresentation::build at a wavefunction;
// orc_frozen_deriv = LayerDerivative of every node at another wavefunction
// with those matrices (node n's result depends on node n's tensor only);
// orc_frozen_rho = the density matrices of the build.  The caller keeps the
// operator and SOP arrays alive for the session's life.
struct Frozen {
  Tree t;
  Ops ops;
  Sop s;
  std::vector<cd> at;
  Sweep* sw = nullptr;
};

void* orc_frozen_new(int backend, int n_nodes, const int* order, const int* dims, const int* parent,
                     const int* child_idx, const int* leaf_mode, int n_ops, const int* op_kind,
                     const int* op_dim, const int64_t* op_off, const double* op_data, int n_terms,
                     const double* coeff, const int* term_ptr, const int* term_mode, const int* term_op,
                     double eps) {
  (void)n_ops;
  Frozen* f = new Frozen;
  f->t = make_tree(n_nodes, order, dims, parent, child_idx, leaf_mode);
  f->ops = Ops{op_kind, op_dim, op_off, (const cd*)op_data};
  f->s = Sop{n_terms, (const cd*)coeff, term_ptr, term_mode, term_op};
  f->at.assign(f->t.off[f->t.n], cd(0));
  f->sw = new Sweep(f->t, f->ops, f->s, (Backend)backend, f->at.data(), eps);
  return f;
}

int orc_frozen_build(void* h, const double* psi) {
  Frozen* f = (Frozen*)h;
  std::memcpy(f->at.data(), psi, sizeof(cd) * f->at.size());
  f->sw->psi = f->at.data();
  f->sw->density();
  f->sw->invert();
  f->sw->represent();
  f->sw->meanfield();
  return 0;
}

int orc_frozen_deriv(void* h, const double* psi, double phase_re, double phase_im, double* out) {
  Frozen* f = (Frozen*)h;
  std::memcpy(f->at.data(), psi, sizeof(cd) * f->at.size());
  f->sw->psi = f->at.data();
  const cd phase(phase_re, phase_im);
  for (int n = 0; n < f->t.n; ++n) f->sw->layer_derivative(n, (cd*)out + f->t.off[n], phase);
  return 0;
}

// LayerDerivative of node n alone, at node tensor phi
int orc_frozen_deriv_node(void* h, int n, const double* phi, double phase_re, double phase_im, double* out) {
  Frozen* f = (Frozen*)h;
  if (n < 0 || n >= f->t.n) return 1;
  std::memcpy(f->at.data() + f->t.off[n], phi, sizeof(cd) * f->t.size[n]);
  f->sw->psi = f->at.data();
  f->sw->layer_derivative(n, (cd*)out, cd(phase_re, phase_im));
  return 0;
}

int orc_frozen_rho(void* h, double* out) {
  Frozen* f = (Frozen*)h;
  std::memcpy(out, f->sw->rho.data(), sizeof(cd) * f->sw->rho.size());
  return 0;
}

void orc_frozen_free(void* h) {
  Frozen* f = (Frozen*)h;
  delete f->sw;
  delete f;
}

// ---------------------------------------------------------------------------
// SCF / Krylov sweep (src/Applications/SCF.cpp:14-341) with the tail-free
// HamiltonianRepresentation and its corrections
// (src/TreeClasses/HamiltonianRepresentation.cpp:117-203), the compiled twin
// of oracle/scf.py (same routines, same order; the products through
// mode_product / hole_product, zgemm when a BLAS is attached).
// ---------------------------------------------------------------------------
struct ScfRep {
  const Tree& t;
  const Ops& ops;
  const Sop& s;
  Backend be;
  int L;
  std::vector<std::vector<char>> stree;        // [term][node], tail-free sparse tree
  std::vector<std::vector<int>> nact;          // [node][term]
  std::vector<std::vector<std::vector<cd>>> hmat, hcon;  // [term][node] d x d
  std::vector<std::vector<cd>> hcorr, hconcorr;          // [node] d x d

  ScfRep(const Tree& t_, const Ops& o_, const Sop& s_, Backend be_) : t(t_), ops(o_), s(s_), be(be_) {
    L = s.n_terms;
    stree.assign(L, std::vector<char>(t.n, 0));
    for (int l = 0; l < L; ++l) {
      // SparseTree without tail (src/TreeClasses/SparseTree.cpp:34-84)
      std::vector<char> path(t.n, 0);
      for (int f = s.ptr[l]; f < s.ptr[l + 1]; ++f)
        for (int a = t.leaf_node.at(s.mode[f]); a >= 0; a = t.parent[a]) path[a] = 1;
      std::vector<int> order;
      for (int a = 0; a < t.n; ++a)
        if (path[a]) order.push_back(a);
      int m = (int)order.size() - 1;
      while (m > 0) {
        int k = 0;
        for (int c : t.children[order[m]]) k += path[c];
        if (k > 1) break;
        --m;
      }
      ++m;
      for (int q = 0; q < m; ++q) stree[l][order[q]] = 1;
    }
    nact.assign(t.n, std::vector<int>(L, 0));
    for (int a = 0; a < t.n; ++a)
      for (int l = 0; l < L; ++l) {
        if (t.bottom(a)) {
          int hit = 0;
          for (int f = s.ptr[l]; f < s.ptr[l + 1]; ++f) hit |= (s.mode[f] == t.leaf_mode[a]);
          nact[a][l] = hit;
          continue;
        }
        int k = 0;
        for (int c : t.children[a]) k += stree[l][c];
        nact[a][l] = t.top(a) ? k : k + stree[l][a];
      }
    hmat.assign(L, std::vector<std::vector<cd>>(t.n));
    hcon.assign(L, std::vector<std::vector<cd>>(t.n));
    for (int l = 0; l < L; ++l)
      for (int a = 0; a < t.n; ++a)
        if (stree[l][a]) {
          hmat[l][a].assign((size_t)t.dup(a) * t.dup(a), cd(0));
          hcon[l][a].assign((size_t)t.dup(a) * t.dup(a), cd(0));
        }
    hcorr.assign(t.n, {});
    hconcorr.assign(t.n, {});
    for (int a = 0; a < t.n; ++a) {
      hcorr[a].assign((size_t)t.dup(a) * t.dup(a), cd(0));
      hconcorr[a].assign((size_t)t.dup(a) * t.dup(a), cd(0));
    }
  }

  // C = h x_k B on node a's geometry
  void mp(std::vector<cd>& C, const std::vector<cd>& h, const std::vector<cd>& B, int a, int k) const {
    C.resize(B.size());
    const int64_t d = t.shape[a][k];
    mode_product(be, C.data(), h.data(), B.data(), t.before(a, k), d, d, t.after(a, k), true);
  }
  // S = contraction of A and B over every index but k
  void hole(std::vector<cd>& S, const std::vector<cd>& A, const std::vector<cd>& B, int a, int k) const {
    const int64_t d = t.shape[a][k];
    S.assign((size_t)d * d, cd(0));
    hole_product(be, S.data(), A.data(), B.data(), t.before(a, k), d, d, t.after(a, k));
  }
  std::vector<cd> leaf_apply(int l, const std::vector<cd>& x, int a) const {
    std::vector<cd> buf(x), tmp(x.size());
    apply_mlo(be, ops, s, l, t.leaf_mode[a], buf.data(), tmp.data(), t.shape[a][0], t.dup(a));
    return buf;
  }
  std::vector<cd> apply_children(int l, const std::vector<cd>& x, int a, int skip) const {
    std::vector<cd> y(x), z;
    for (size_t k = 0; k < t.children[a].size(); ++k) {
      const int c = t.children[a][k];
      if ((int)k == skip || !stree[l][c]) continue;
      mp(z, hmat[l][c], y, a, (int)k);
      y.swap(z);
    }
    return y;
  }
  static void axpy(std::vector<cd>& y, cd a, const std::vector<cd>& x) {
    for (size_t i = 0; i < y.size(); ++i) y[i] += a * x[i];
  }

  void build_up(const std::vector<std::vector<cd>>& psi, int a) {
    const std::vector<cd>& phi = psi[a];
    const int last = t.last(a);
    for (int l = 0; l < L; ++l) {
      if (!stree[l][a]) continue;
      hole(hmat[l][a], phi, t.bottom(a) ? leaf_apply(l, phi, a) : apply_children(l, phi, a, -1), a, last);
    }
    // buildUpCorrection
    const int d = t.dup(a);
    std::vector<cd> corr((size_t)d * d, cd(0)), z;
    if (!t.bottom(a)) {
      std::vector<cd> hA(phi.size(), cd(0));
      for (size_t k = 0; k < t.children[a].size(); ++k) {
        mp(z, hcorr[t.children[a][k]], phi, a, (int)k);
        axpy(hA, cd(1), z);
      }
      hole(corr, phi, hA, a, last);
    }
    if (!t.top(a)) {
      const int p = t.parent[a];
      for (int l = 0; l < L; ++l)
        if (nact[p][l] == 1 && stree[l][a]) axpy(corr, s.coeff[l], hmat[l][a]);
    }
    hcorr[a] = corr;
  }

  void build_down(const std::vector<std::vector<cd>>& psi, int a) {
    if (t.top(a)) return;
    const int p = t.parent[a];
    const std::vector<cd>& phi = psi[p];
    const int plast = t.last(p), ci = t.child_idx[a];
    std::vector<cd> z;
    for (int l = 0; l < L; ++l) {
      if (!stree[l][a]) continue;
      std::vector<cd> x = apply_children(l, phi, p, ci);
      if (!t.top(p) && stree[l][p]) {
        mp(z, hcon[l][p], x, p, plast);
        x.swap(z);
      }
      hole(hcon[l][a], phi, x, p, ci);
    }
    // buildDownCorrection(hole = a)
    std::vector<cd> hA(phi.size(), cd(0));
    for (int l = 0; l < L; ++l) {
      if (nact[p][l] < 2 || stree[l][a]) continue;
      std::vector<cd> x = apply_children(l, phi, p, ci);
      if (!t.top(p) && stree[l][p]) {
        mp(z, hcon[l][p], x, p, plast);
        x.swap(z);
      }
      axpy(hA, s.coeff[l], x);
    }
    for (size_t k = 0; k < t.children[p].size(); ++k) {
      if ((int)k == ci) continue;
      mp(z, hcorr[t.children[p][k]], phi, p, (int)k);
      axpy(hA, cd(1), z);
    }
    if (!t.top(p)) {
      mp(z, hconcorr[p], phi, p, plast);
      axpy(hA, cd(1), z);
    }
    hole(hconcorr[a], phi, hA, p, ci);
  }

  // effective Hamiltonian at node a (SCF.cpp:36-84)
  std::vector<cd> apply(const std::vector<cd>& A, int a) const {
    const int last = t.last(a);
    std::vector<cd> HA(A.size(), cd(0)), z;
    for (int l = 0; l < L; ++l) {
      if (t.bottom(a)) {
        if (stree[l][a]) {
          mp(z, hcon[l][a], leaf_apply(l, A, a), a, last);
          axpy(HA, s.coeff[l], z);
        }
      } else if (nact[a][l] > 1) {
        std::vector<cd> x = apply_children(l, A, a, -1);
        if (!t.top(a) && stree[l][a]) {
          mp(z, hcon[l][a], x, a, last);
          x.swap(z);
        }
        axpy(HA, s.coeff[l], x);
      }
    }
    if (!t.bottom(a))
      for (size_t k = 0; k < t.children[a].size(); ++k) {
        mp(z, hcorr[t.children[a][k]], A, a, (int)k);
        axpy(HA, cd(1), z);
      }
    if (!t.top(a)) {
      mp(z, hconcorr[a], A, a, last);
      axpy(HA, cd(1), z);
    }
    return HA;
  }
};

static cd vdot(const std::vector<cd>& a, const std::vector<cd>& b) {
  cd acc = 0;
  for (size_t i = 0; i < a.size(); ++i) acc += std::conj(a[i]) * b[i];
  return acc;
}

// thin Householder QR of node a's tensor with index `mode` as the column
// index (toMatrix / qr / toTensor, include/Core/Tensor_Implementation.h:863-869)
static std::vector<cd> qr_mode(const Tree& t, int a, const std::vector<cd>& x, int mode) {
  const int64_t before = t.before(a, mode), C = t.shape[a][mode], after = t.after(a, mode);
  const int64_t R = before * after;
  std::vector<cd> M((size_t)(R * C));
  for (int64_t aft = 0; aft < after; ++aft)
    for (int64_t c = 0; c < C; ++c)
      for (int64_t b = 0; b < before; ++b) M[(b + before * aft) + R * c] = x[b + before * (c + C * aft)];
  // Householder: M = H_0 .. H_{C-1} [R; 0]
  std::vector<std::vector<cd>> V(C);
  std::vector<cd> tau(C, cd(0));
  for (int64_t j = 0; j < C; ++j) {
    double nrm2 = 0;
    for (int64_t i = j; i < R; ++i) nrm2 += std::norm(M[i + R * j]);
    const double nrm = std::sqrt(nrm2);
    const cd x0 = M[j + R * j];
    const double ax0 = std::abs(x0);
    const cd ph = ax0 > 0 ? x0 / ax0 : cd(1);
    const cd alpha = -ph * nrm;
    std::vector<cd> v(R - j);
    for (int64_t i = j; i < R; ++i) v[i - j] = M[i + R * j];
    v[0] -= alpha;
    double vn = 0;
    for (auto& e : v) vn += std::norm(e);
    if (vn > 0) {
      tau[j] = 2.0 / vn;
      for (int64_t k = j; k < C; ++k) {
        cd w = 0;
        for (int64_t i = j; i < R; ++i) w += std::conj(v[i - j]) * M[i + R * k];
        w *= tau[j];
        for (int64_t i = j; i < R; ++i) M[i + R * k] -= v[i - j] * w;
      }
    }
    V[j] = v;
  }
  // Q = H_0 .. H_{C-1} [I; 0]
  std::vector<cd> Q((size_t)(R * C), cd(0));
  for (int64_t j = 0; j < C; ++j) Q[j + R * j] = 1.0;
  for (int64_t j = C - 1; j >= 0; --j) {
    if (tau[j] == cd(0)) continue;
    for (int64_t k = 0; k < C; ++k) {
      cd w = 0;
      for (int64_t i = j; i < R; ++i) w += std::conj(V[j][i - j]) * Q[i + R * k];
      w *= tau[j];
      for (int64_t i = j; i < R; ++i) Q[i + R * k] -= V[j][i - j] * w;
    }
  }
  std::vector<cd> out(x.size());
  for (int64_t aft = 0; aft < after; ++aft)
    for (int64_t c = 0; c < C; ++c)
      for (int64_t b = 0; b < before; ++b) out[b + before * (c + C * aft)] = Q[(b + before * aft) + R * c];
  return out;
}

int orc_scf(int backend, int n_nodes, const int* order, const int* dims, const int* parent,
            const int* child_idx, const int* leaf_mode, int n_ops, const int* op_kind, const int* op_dim,
            const int64_t* op_off, const double* op_data, int n_terms, const double* coeff,
            const int* term_ptr, const int* term_mode, const int* term_op, double* psi_io, int n_iter,
            int n_krylov, int n_itp, double beta, double breakdown, double* energies, int64_t cap,
            int64_t* count) {
  (void)n_ops;
  Tree t = make_tree(n_nodes, order, dims, parent, child_idx, leaf_mode);
  Ops ops{op_kind, op_dim, op_off, (const cd*)op_data};
  Sop s{n_terms, (const cd*)coeff, term_ptr, term_mode, term_op};
  cd* flat = (cd*)psi_io;
  std::vector<std::vector<cd>> psi(t.n);
  for (int a = 0; a < t.n; ++a) psi[a].assign(flat + t.off[a], flat + t.off[a] + t.size[a]);
  ScfRep rep(t, ops, s, (Backend)backend);
  for (int a = 0; a < t.n; ++a)
    if (!t.top(a)) rep.build_up(psi, a);
  // sweep order: depth first from the top, back to a node after each child
  std::vector<int> ord;
  std::function<void(int)> add = [&](int a) {
    ord.push_back(a);
    for (int c : t.children[a]) {
      add(c);
      ord.push_back(a);
    }
  };
  add(t.n - 1);
  auto adjacent = [&](int frm, int to) -> int {
    if (to < 0) return t.last(frm);
    for (size_t k = 0; k < t.children[frm].size(); ++k)
      if (t.children[frm][k] == to) return (int)k;
    return t.last(frm);
  };
  int64_t ne = 0;
  for (int it = 0; it < n_iter; ++it) {
    for (size_t i = 0; i < ord.size(); ++i) {
      const int a = ord[i];
      int size = (int)std::min<int64_t>(n_krylov, t.size[a]);
      // solveKrylovSpace (SCF.cpp:138-195)
      std::vector<std::vector<cd>> space;
      std::vector<double> al, be;
      std::vector<cd> x = psi[a];
      {
        const double nx = std::sqrt(vdot(x, x).real());
        for (auto& e : x) e /= nx;
      }
      space.push_back(x);
      std::vector<cd> hx = rep.apply(x, a);
      al.push_back(vdot(x, hx).real());
      for (size_t q = 0; q < x.size(); ++q) x[q] = hx[q] - al.back() * x[q];
      for (int l = 1; l < size; ++l) {
        const double nrm = std::sqrt(vdot(x, x).real());
        if (breakdown >= 0) {
          double sc = 0;
          for (double v : al) sc = std::max(sc, std::fabs(v));
          for (double v : be) sc = std::max(sc, v);
          if (nrm <= breakdown * sc) break;
        }
        be.push_back(nrm);
        for (auto& e : x) e /= nrm;
        space.push_back(x);
        hx = rep.apply(x, a);
        al.push_back(vdot(x, hx).real());
        for (size_t q = 0; q < x.size(); ++q) x[q] = hx[q] - al.back() * space[l][q] - be.back() * space[l - 1][q];
      }
      size = (int)al.size();
      std::vector<cd> T((size_t)size * size, cd(0)), U((size_t)size * size);
      std::vector<double> E(size);
      for (int l = 0; l < size; ++l) T[l + size * l] = al[l];
      for (int l = 0; l + 1 < size; ++l) T[(l + 1) + size * l] = T[l + size * (l + 1)] = be[l];
      herm_eig(size, T.data(), U.data(), E.data());
      if (energies && ne < cap) energies[ne] = E[0];
      ++ne;
      std::vector<cd> w(t.size[a], cd(0));
      if (it < n_itp) {
        // imaginaryTimePropagation: the k = 0 term enters twice (SCF.cpp:208-214)
        for (int l = 0; l < size; ++l) {
          cd c = U[l] * std::conj(U[0]);
          for (int k = 0; k < size; ++k) c += U[l + size * k] * std::exp(-beta * (E[k] - E[0])) * std::conj(U[size * k]);
          ScfRep::axpy(w, c, space[l]);
        }
        const double nw = std::sqrt(vdot(w, w).real());
        for (auto& e : w) e /= nw;
      } else {
        for (int l = 0; l < size; ++l) ScfRep::axpy(w, U[l], space[l]);
      }
      const int nxt = i + 1 < ord.size() ? ord[i + 1] : -1;
      const int out_idx = adjacent(a, nxt);
      psi[a] = qr_mode(t, a, w, out_idx);
      if (nxt < 0) break;
      std::vector<cd> r, z;
      rep.hole(r, psi[a], w, a, out_idx);
      const int in_idx = adjacent(nxt, a);
      rep.mp(z, r, psi[nxt], nxt, in_idx);
      psi[nxt] = z;
      if (!t.top(a) && t.parent[a] == nxt)
        rep.build_up(psi, a);
      else
        rep.build_down(psi, nxt);
    }
  }
  for (int a = 0; a < t.n; ++a) std::copy(psi[a].begin(), psi[a].end(), flat + t.off[a]);
  if (count) *count = ne;
  return 0;
}

}  // extern "C"
