// qt_internal.h -- types shared by the planner (qt_plan.cpp), the kernels
// (qt_kernels.cu) and the C ABI (qt_api.cu) of libqtgpu.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <map>
#include <string>
#include <vector>

namespace qt {

// ---------------------------------------------------------------------------
// Device task records.  One record describes one tensor operation; a launch
// ("stage") runs a contiguous range of records, split into tiles.
// ---------------------------------------------------------------------------

// Mode-k product: out[b, j, c] = alpha * sum_a h(j, a) in[b, a, c]
// (h is a_out x a_in, column-major).  diag != 0: h is the diagonal of a
// leaf operator (length a_in == a_out) and out[b, j, c] = alpha*h[j]*in[b,j,c].
// out must not alias in.
struct MPTask {
  const double2* in;
  double2* out;
  const double2* h;
  double2 alpha;
  int before, a_in, a_out, after;
  int diag;
  int add;  // 1: out += result
  void* oz_h = nullptr;  // tensor-core path: digits of h (written by the stage's pre-pass)
};

// Hole product: S(i, j) = sum_{b, c} conj(A[b, i, c]) * B[b, j, c].
struct HPTask {
  const double2* A;
  const double2* B;
  double2* S;
  int before, a, after;
  int aB;      // columns of S (activeB); 0 means aB == a
  int splits;  // k ranges of kchunk rows; > 1: partial tiles go to the workspace
  int kchunk;
  int64_t ws;  // workspace offset (elements) of the partial tiles
  int rows, cols;  // outputs per thread along i and j (1..4)
};

// hole products on the tensor cores (qt_umma.cu, double-float plans): groups
// of up to eight tasks that share the operand A form one 128-row accumulator
// tile (rows: the tasks' B columns j, columns: A's i, real and imaginary
// parts); the reduction runs in chunks of hp_tc_kc(ap) k, each chunk with
// its own power-of-two scales.  A group's member tasks (indices into the task table)
// all have the same a, before and after.
constexpr int kHpTcChunk = 64;     // k of the shorter chunks
constexpr int kHpTcMembers = 8;    // tasks per group (a >= 16)
struct HpTcGroup {
  const double2* A;
  unsigned char* img;  // A's operand images, one per chunk of hp_tc_kc(ap) k
  unsigned char* ex;   // biased row exponents of the members' B, 128 rows per chunk
  int before, a, after;
  int ap;              // a padded to a multiple of 8
  int n, nchunks;
  int member[kHpTcMembers];
};
// Which contractions the planner puts on the tensor cores: shapes from a
// lower bound per kind to 64 (padded to at most 64 output columns).  Below
// the bound the fixed costs of a tile (row exponents, the level
// recombination, the 128-row tile itself) outweigh the products.  The
// default bounds, 32, were measured on a forest of uneven trees with bonds
// 4..24: the double-float sweep took 82.7 ms with every shape up to 64 on the
// tensor cores, 57.2 ms with the bounds (as on the FP32 pipe alone);
// qt_set_tc_thresholds takes bounds found by the autotuner
// (qutree_gb300/autotune.py).  65 keeps a kind off the tensor cores.
struct TcTune {
  int mp = 32, hp = 32, acc = 32;
};
// hole product: lo <= a <= 64 and at least two 64-k chunks of reduction
inline bool hp_tc_eligible(int before, int a, int after, int lo = 32) {
  return a >= lo && a <= 64 && (int64_t)before * after >= 2 * kHpTcChunk;
}
// mode product (not diagonal): lo <= a_in, a_out <= 64
inline bool mp_tc_eligible(int a_in, int a_out, int lo = 32) {
  return a_in >= lo && a_in <= 64 && a_out >= lo && a_out <= 64;
}
#ifdef __CUDACC__
#define QT_HD __host__ __device__
#else
#define QT_HD
#endif
// reduction length of a chunk: 128 k for ap > 32, whose four level
// accumulators keep the levels 0..2 exact up to 170 k, else 64 k (seven
// exact levels up to 73 k)
QT_HD constexpr int hp_tc_kc(int ap) { return ap > 32 ? 2 * kHpTcChunk : kHpTcChunk; }
// bytes of one unit's operand image: steps of 16 k x 7 digits x rows
// [-Wi | Wr | Wi] (3 ap) x 16 bf16, then the column exponents (int, 64 slots)
QT_HD constexpr int64_t hp_tc_chunk_bytes(int ap, int steps) {
  return (int64_t)steps * 7 * 3 * ap * 16 * 2 + 64 * 4;
}

// out[r, j] (+)= alpha * sum_t sum_j' H_t(j, j') X_t[r, j'] over the terms
// [first, first+count) of the AccTerm table; H == nullptr means identity.
struct AccTerm {
  const double2* H;
  const double2* X;
};
struct AccTask {
  double2* out;
  const double2* alpha_ptr;  // if non-null, alpha is read from device memory
  double2 alpha;
  int rows, d;
  int first, count;
  int add, pad;
  void* tc_img = nullptr;  // tensor-core path: images of alpha H_t, one per term (hp_tc_chunk_bytes(., 4))
};
// an accumulation the planner puts on the tensor cores (double-float plans):
// lo <= d <= 64 and at least 64 rows
inline bool acc_tc_eligible(int rows, int d, int lo = 32) { return d >= lo && d <= 64 && rows >= 64; }

// out = sum_t c_t * M_t for d x d matrices (grouped mean fields).
struct LinTerm {
  double2 c;
  const double2* M;
};
struct LinTask {
  double2* out;
  int d, first, count, pad;
};

// out = sum_t A_t op(B_t) for d x d matrices, op(B) = B^T when trans_b
// (the small matrix products of the fused derivative).
struct MMTerm {
  const double2* A;
  const double2* B;
};
struct MMTask {
  double2* out;
  int d, first, count, trans_b;
};

// Regularised inverse of a Hermitian d x d matrix via Jacobi eigensolver.
struct EigTask {
  const double2* rho;
  double2* rhoinv;
  double2* U;  // d x d scratch
  int d, pad;
};

// Per non-top node: Sinv = S^-1, P = Sinv * D, M2 = -(rhoinv * P^T).
struct ProjTask {
  double2* S;  // overwritten (Gauss-Jordan work)
  const double2* D;
  const double2* rhoinv;
  double2* Sinv;
  double2* P;
  double2* M2;
  int d, pad;
};

// Elementwise precision conversion of n complex numbers: dir 0 complex128 ->
// double-float (float4 hi/lo pairs), dir 1 double-float -> complex128.
struct CvtTask {
  const void* src;
  void* dst;
  int64_t n;
  int dir, pad;
};

// Energy-gradient preparation per node (orthonormal gauge):
//   M3 = Eout - E * rho,  E = Re h00 / Re S00 of the node's tree,
// and, on the tree's root task, alpha = 1 / Re S00 (complex128).
struct GradTask {
  const double2* eout;  // d x d, nullptr for a root (zero environment)
  const double2* rho;   // d x d
  double2* m3;          // d x d
  const double2* h00;   // complex128 <Phi_top|H Phi_top> of the tree
  const double2* s00;   // complex128 <Phi_top|Phi_top> of the tree
  double2* alpha;       // complex128 1/S00, written when write_alpha != 0
  int d, write_alpha;
};

// ---- CDVR (potential on time-dependent grids) -----------------------------
// Strided complex contraction, the workhorse of the CDVR stages:
//   C[m, n] = alpha * sum_k opA(A)[m, k] opB(B)[k, n]  (+ C[m, n] when add)
// with two-level indices m = (m0, m1), n = (n0, n1), k = (k0, k1); the
// element of A at (m, k) sits at m0*am0 + m1*am1 + k0*ak0 + k1*ak1 (B, C
// alike).  opX conjugates when conjX.  Covers mode products (plain,
// transposed, adjoint matrices), hole products, double-hole contractions,
// the d^4 x d^2 corrections and matrix products.
struct TCTask {
  const double2* A;
  const double2* B;
  double2* C;
  double2 alpha;
  int M0, M1, N0, N1, K0, K1;
  int conjA, conjB, add, pad;
  int64_t am0, am1, ak0, ak1;
  int64_t bk0, bk1, bn0, bn1;
  int64_t cm0, cm1, cn0, cn1;
};
constexpr int kTcTile = 32;  // output tile (kTcTile x kTcTile) of one block

// out = gramSchmidt(in + noise) on the (rows x cols) matrix view of a node
struct GSTask {
  const double2* in;
  const double2* noise;
  double2* out;
  int rows, cols;
};

// Spectral function of a Hermitian d x d matrix: out = U f(lambda) U^dagger.
// fn: 0 regularised inverse 1/(l + eps e^(-l/eps)); 1 sqrt(max(l, 0));
// 2 regularised inverse of the square root (g = sqrt(max(l, 0)));
// 3 regularised square root g + eps e^(-g/eps); 4 eigenvectors only:
// out = U^dagger and vals = ascending eigenvalues (real parts).
struct EigFTask {
  const double2* A;
  double2* out;
  double2* U;     // d x d scratch
  double2* W;     // d x d scratch
  double2* vals;  // fn 4: d eigenvalues
  double eps;
  int d, fn;
};

// Weighted simultaneous diagonalisation of n Hermitian matrices with weight
// W (LayerGrid with several matrices): trafo = T^dagger, grid = n x d values;
// scratch holds 2n + 2 matrices.  The matrices are terms [first, first + n).
struct WSDTask {
  const double2* W;
  double2* trafo;
  double2* grid;
  double2* scratch;
  int d, n, first, pad;
};
struct WSDTerm {
  const double2* X;
};

// Potential on a grid tensor: element (i_0, ..., i_{order-1}) gets
// V(x) with x_g = Re grid_g[i_{index_g}] for the f coordinates g
// (coords [first, first + f)).  V is the polynomial term table.
struct VCoord {
  const double2* grid;
  int index, pad;
};
struct VPotTask {
  double2* out;
  int64_t n;
  int order, first;
  int dims[6];
};
struct PotTerm {
  double c;
  int first, count;  // factors [first, first + count)
};
struct PotFactor {
  int mode, power;
};

// Local part of the CDVR correction tensor of an edge:
//   dv(l1, i0, m1, i0) = sum_b conj(cup(b, l1)) vnode(b, i0) cup(b, m1),
//   dv(l0, l1, l0, l1) -= vedge(l0, l1), zero elsewhere.
struct DVLTask {
  const double2* cup;
  const double2* vnode;
  const double2* vedge;
  double2* dv;
  int bef, d;
};

// out[i] = (add ? out[i] : 0) + v[i] * in[i]
struct EWTask {
  const double2* v;
  const double2* in;
  double2* out;
  int64_t n;
  int add, pad;
};

enum StageKind {
  ST_MP = 0, ST_HP, ST_ACC, ST_LIN, ST_EIG, ST_PROJ, ST_CVT, ST_GRAD, ST_MM,
  ST_TC, ST_GS, ST_EIGF, ST_WSD, ST_VPOT, ST_DVL, ST_EW
};

struct Stage {
  int kind;
  int64_t first_task, n_tasks;
  int64_t first_tile, n_tiles;
  const char* name;
  int aux = 0;       // hole-product stage with split tasks: a second kernel sums the partial tiles
  int seg0 = 0, nseg = 0;  // hole-product stage: its tile segments (one launch per micro-tile shape)
  int64_t oz0 = 0, noz = 0;  // mode-product stage: its tensor-core tiles (mp_oz_tiles)
  int64_t ozt0 = 0, nozt = 0;  // and its tensor-core tasks (mp_oz_tasks, digits of h)
  int64_t hti0 = 0, nhti = 0;  // hole-product stage: its tensor-core items (hp_tc_items)
  int64_t htu0 = 0, nhtu = 0;  // and the units of its image pre-pass (hp_tc_imgs)
  int64_t ati0 = 0, nati = 0;  // accumulation stage: its tensor-core items (acc_tc_items)
  int64_t atu0 = 0, natu = 0;  // and the units of its image pre-pass (acc_tc_imgs)
  int64_t atc_units = 0;       // units (terms) of all its items
  double flops = 0;  // executed flops of the stage
  double bytes = 0;  // algorithmic bytes: operands read once, results written once
};

// ---------------------------------------------------------------------------
// Host-side plan (symbolic; pointers are bound after the arena exists)
// ---------------------------------------------------------------------------
// B_PSI64 / B_DPSI64: the caller-facing complex128 wavefunction and derivative.
// With complex128 arithmetic they alias B_PSI / B_DPSI; with double-float
// arithmetic B_PSI / B_HPHI / B_DPSI hold double-float numbers and conversion
// stages move data across.
// B_GRAD / B_GRAD64: energy gradient (arithmetic format / caller-facing
// complex128; aliases with complex128 arithmetic), only when requested.
// B_KEEP: node-sized tensors the compressed plan keeps from represent to
// Apply (chain outputs and Phi x_last rho).
// B_HPW: partial tiles of hole products split over their reduction index.
// B_KRY: input and output tensor of the SCF effective Hamiltonian (2 x the
// largest node).
// B_CDVR: everything of the CDVR potential (grids, transformations, node and
// edge potentials, correction tensors, their scratch and constants).
enum Buf {
  B_PSI = 0, B_HPHI, B_DPSI, B_MATS, B_OPS, B_SCR, B_PARAM, B_PSI64, B_DPSI64, B_GRAD, B_GRAD64, B_KEEP, B_HPW, B_KRY,
  B_CDVR, B_OZ, B_NBUF
};

struct Ref {
  int buf = -1;
  int64_t off = 0;  // in complex (double2) elements
};

struct NodeGeo {
  std::vector<int> shape;
  int parent = -1, child_idx = -1, leaf_mode = -1;
  std::vector<int> children;
  int64_t N = 0, off = 0;  // elements; packed offset of the node tensor
  int64_t aoff = 0;        // aligned arena offset
  int depth = 0, height = 0;
  int dup() const { return shape.back(); }
  int last() const { return (int)shape.size() - 1; }
  bool top() const { return parent < 0; }
  bool bottom() const { return leaf_mode >= 0; }
  int64_t before(int k) const {
    int64_t b = 1;
    for (int i = 0; i < k; ++i) b *= shape[i];
    return b;
  }
  int64_t after(int k) const {
    int64_t a = 1;
    for (size_t i = k + 1; i < shape.size(); ++i) a *= shape[i];
    return a;
  }
};

struct PlanStats {
  double ref_flops = 0, exec_flops = 0;
  int64_t launches = 0, arena_bytes = 0, scratch_bytes = 0;
  int64_t rep_chains = 0, mf_chains = 0, app_chains = 0;
};

struct Plan {
  // geometry
  std::vector<NodeGeo> nodes;
  int64_t psi_packed = 0, psi_arena = 0;
  // matrices arena layout
  // complex128 copies (rho64 ... m2_64) alias the plain offsets when prec == 0
  std::vector<int64_t> rho_off, rhoinv_off, u_off, s_off, sinv_off, d_off, p_off, m2_off;
  std::vector<int64_t> rho64_off, rhoinv64_off, s64_off, d64_off, m2_64_off;
  // per tree (root) of the forest, in ascending address order
  std::vector<int> tops;
  std::vector<int64_t> energy_off, stop_off;          // complex128 results read by qt_energy
  std::vector<int64_t> energy_dev_off, stop_dev_off;  // written by the hole products
  int prec = 0;
  // per term: its active nodes (ascending) and their represent / mean-field
  // slot offsets (-2: the top's represent matrix, zero by definition)
  std::vector<std::vector<int>> term_nodes;
  std::vector<std::vector<int64_t>> term_hslot, term_cslot;
  bool per_term_mats = true;  // false: the compressed plan keeps no per-term matrices
  int64_t mats_size = 0;
  int64_t scratch_size = 0;
  int64_t keep_size = 0;
  int64_t hpw_size = 0;
  int64_t ops_size = 0;
  // symbolic task lists (buffer-relative); bound to pointers by bind()
  struct SMP {
    Ref in, out, h;
    double2 alpha;
    int before, a_in, a_out, after, diag;
    int64_t oz_h = -1;  // tensor-core path: offset (bytes) of the digits of h in B_OZ
  };
  struct SHP {
    Ref A, B, S;
    int before, a, after;
    int splits = 1, kchunk = 0;
    int64_t ws = 0;
    int rows = 4, cols = 4;
  };
  struct SAccTerm {
    Ref H;  // buf == -1: identity
    Ref X;
  };
  struct SAcc {
    Ref out;
    Ref alpha_ref;  // device scalar (complex128) read as alpha when set
    bool alpha_param;
    double2 alpha;
    int rows, d, first, count, add;
    int64_t tc_img = -1;  // tensor-core path: byte offset of the term images in B_OZ
  };
  struct SLinTerm {
    double2 c;
    Ref M;
  };
  struct SLin {
    Ref out;
    int d, first, count;
  };
  struct SEig {
    Ref rho, rhoinv, U;
    int d;
  };
  struct SProj {
    Ref S, D, rhoinv, Sinv, P, M2;
    int d;
  };
  struct SCvt {
    Ref src, dst;
    int64_t n;
    int dir;
  };
  std::vector<SMP> mp;
  std::vector<SHP> hp;
  std::vector<SAcc> acc;
  std::vector<SAccTerm> acc_terms;
  std::vector<SLin> lin;
  std::vector<SLinTerm> lin_terms;
  std::vector<SEig> eig;
  std::vector<SProj> proj;
  std::vector<SCvt> cvt;
  struct SGrad {
    Ref eout, rho, m3, h00, s00, alpha;
    int d, write_alpha;
  };
  std::vector<SGrad> grad;
  struct SMMTerm {
    Ref A, B;
  };
  struct SMM {
    Ref out;
    int d, first, count, trans_b;
  };
  std::vector<SMM> mm;
  std::vector<SMMTerm> mm_terms;
  // CDVR stages (symbolic)
  struct STC {
    Ref A, B, C;
    double2 alpha;
    int M0, M1, N0, N1, K0, K1;
    int conjA, conjB, add;
    int64_t am0, am1, ak0, ak1, bk0, bk1, bn0, bn1, cm0, cm1, cn0, cn1;
  };
  struct SGS {
    Ref in, noise, out;
    int rows, cols;
  };
  struct SEigF {
    Ref A, out, U, W, vals;
    double eps;
    int d, fn;
  };
  struct SWSD {
    Ref W, trafo, grid, scratch;
    int d, n, first;
  };
  struct SVCoord {
    Ref grid;
    int index;
  };
  struct SVPot {
    Ref out;
    int64_t n;
    int order, first;
    int dims[6];
  };
  struct SDVL {
    Ref cup, vnode, vedge, dv;
    int bef, d;
  };
  struct SEW {
    Ref v, in, out;
    int64_t n;
    int add;
  };
  std::vector<STC> tc;
  std::vector<int4> tc_tiles;  // (task, m tile, n tile, 0)
  std::vector<SGS> gs;
  std::vector<SEigF> eigf;
  std::vector<SWSD> wsd;
  std::vector<Ref> wsd_terms;
  std::vector<SVPot> vpot;
  std::vector<SVCoord> vcoords;
  std::vector<int2> vpot_tiles;  // (task, first element)
  std::vector<SDVL> dvl;
  std::vector<int2> dvl_tiles;
  std::vector<SEW> ew;
  std::vector<int2> ew_tiles;
  bool cdvr = false;
  int64_t cdvr_size = 0;
  int wsd_max_n = 0, wsd_max_d = 0;  // largest joint-diagonalisation problem
  // constant contents of B_CDVR written at prepare (offset, values)
  std::vector<std::pair<int64_t, std::vector<double2>>> cdvr_init;
  // offsets of the CDVR quantities (per node; -1 where absent)
  struct CdvrLayout {
    // per node (-1 where absent)
    std::vector<int64_t> noise, chi, at, cup, cdown, vnode, xi, vx, tmpa, tmpb;
    std::vector<int64_t> rho_chi, isq, trafo, htrafo, sqrt_rho, binv, g, sqrho, lm, edge1, edges,
        vedge, dv;
    std::vector<int64_t> grid, hgrid;  // grid values of the node / hole problem (n x d)
    std::vector<std::vector<int>> grid_modes, hole_modes;  // X-matrix modes of the two problems
    std::vector<std::vector<int64_t>> xmat, xhole_raw, xhole, xt;  // [mode][node]
    std::vector<int64_t> leafx;  // per mode: its DVR grid (complex, real part)
    std::vector<std::vector<int64_t>> corr_x, corr_y;  // [node][child]: hole and corrected matrix of apply
    int64_t identity_top = -1;
  } cd;
  int64_t cdvr_update_begin = 0, cdvr_update_end = 0;  // stage range of CDVR::Update
  std::vector<int2> mm_tiles;  // (task, first output element), 256 outputs per tile
  bool want_grad = false;
  std::vector<Stage> stages;
  // stages [0, apply_begin) build the matrices (HamiltonianRepresentation::
  // build); stages [apply_begin, end) are LayerDerivative at every node with
  // those matrices frozen.  With double-float arithmetic stage 0 converts Psi.
  int64_t apply_begin = 0;
  // stages [0, main_end) are the sweep.  Stages [main_end, end), when present,
  // replace [apply_begin, main_end) in the frozen-matrix derivative graph.
  int64_t main_end = 0;
  // SCF (QT_PLAN_SCF): per node the stage ranges [begin, end) of buildUp,
  // buildDown and the effective Hamiltonian (B_KRY input at kry_in, output at
  // kry_out); empty ranges where the reference does nothing
  bool scf = false;
  std::vector<int64_t> scf_up_b, scf_up_e, scf_down_b, scf_down_e, scf_apply_b, scf_apply_e;
  int64_t kry_in = 0, kry_out = 0, kry_size = 0;
  // tiles (bound with task indices only)
  std::vector<int2> mp_tiles;
  std::vector<int4> hp_tiles;
  std::vector<int4> hp_segs;  // (rows, cols, first tile, tile count) per hole-product launch
  // double-float plans with tensor-core mode products: (task, block of 32 rows)
  bool mp_tensor = false;
  std::vector<int2> mp_oz_tiles;
  std::vector<int> mp_oz_tasks;
  int64_t oz_bytes = 0;  // B_OZ: operand images of the tensor-core tasks of one stage (reused by every stage)
  // double-float plans with tensor-core hole products (groups bound to HpTcGroup)
  bool hp_tensor = false;
  TcTune tune;  // the tensor-core bounds the plan was built with
  struct SHpTcGroup {
    Ref A;
    int before = 0, a = 0, after = 0, n = 0, nchunks = 0;
    int member[kHpTcMembers] = {0, 0, 0, 0, 0, 0, 0, 0};
    int64_t img = 0;  // byte offset of the images in B_OZ
    int64_t ex = 0;   // byte offset of the row exponents in B_OZ (128 per chunk)
  };
  std::vector<SHpTcGroup> hp_tc_groups;
  std::vector<int4> hp_tc_items;  // (group, z, first chunk, end chunk)
  std::vector<int2> hp_tc_imgs;   // (group, chunk) of the image pre-pass
  std::vector<int4> acc_tc_items;  // (task, 128-row block, units before the item in its stage, 0)
  std::vector<int2> acc_tc_imgs;   // (task, term) of the image pre-pass
  std::vector<int4> acc_tiles;
  std::vector<int2> cvt_tiles;
  // constant matrices written once at prepare: (offset, d) identity
  std::vector<std::pair<int64_t, int>> identities;
  PlanStats stats;
  int max_eig_d = 0;
};

struct OpTable {
  std::vector<int> kind, dim;
  std::vector<int64_t> off;
  std::vector<double> data;  // interleaved
};

struct SopDesc {
  int n_terms = 0;
  std::vector<double2> coeff;
  std::vector<int> ptr, mode, op;
};

// Potential of a Hamiltonian with hasV (CDVR): the DVR grid of every leaf
// (per mode, its leaf dimension) and a polynomial V(x) = sum_t c_t prod x_g^p.
struct CdvrDesc {
  std::vector<std::vector<double>> leaf_x;
  std::vector<double> coeff;
  std::vector<int> ptr, mode, power;
  bool aligned = false;  // hole grids by mode instead of the reference's rank order
};

// CDVR stages (qt_cdvr_plan.cpp): part 0 lays out B_CDVR and emits the
// stages of CDVR::Update, part 1 the stages of CDVR::apply that add to
// B_HPHI.  Returns the executed flops of the emitted stages.
double cdvr_plan(Plan& P, const CdvrDesc& D, int part);

// planner entry point; returns "" on success or an error message
// flavour: 0 reference call sequence, 1 grouped; prec: 0 complex128, 1 double-float;
// grad: also compute the energy gradient with respect to every node tensor
// cdvr: the potential of a Hamiltonian with hasV (nullptr: pure SOP)
// tune: the tensor-core bounds per kind
std::string build_plan(Plan& plan, const std::vector<NodeGeo>& nodes, const OpTable& ops,
                       const SopDesc& sop, int flavour, int prec, int64_t scratch_budget_elems,
                       bool grad = false, const CdvrDesc* cdvr = nullptr, const TcTune& tune = TcTune());

// kernel launches (qt_kernels.cu)
struct DevTables {
  MPTask* mp = nullptr;
  HPTask* hp = nullptr;
  AccTask* acc = nullptr;
  AccTerm* acc_terms = nullptr;
  LinTask* lin = nullptr;
  LinTerm* lin_terms = nullptr;
  EigTask* eig = nullptr;
  ProjTask* proj = nullptr;
  int2* mp_tiles = nullptr;
  int4* hp_tiles = nullptr;
  int4* acc_tiles = nullptr;
  CvtTask* cvt = nullptr;
  int2* cvt_tiles = nullptr;
  GradTask* grad = nullptr;
  void* hp_ws = nullptr;
  MMTask* mm = nullptr;
  MMTerm* mm_terms = nullptr;
  int2* mm_tiles = nullptr;
  const int4* hp_segs = nullptr;  // host array: (rows, cols, first tile, tile count)
  int2* mp_oz_tiles = nullptr;
  int* mp_oz_tasks = nullptr;
  HpTcGroup* hp_tc_groups = nullptr;
  int4* hp_tc_items = nullptr;
  int2* hp_tc_imgs = nullptr;
  int4* acc_tc_items = nullptr;
  int2* acc_tc_imgs = nullptr;
  TCTask* tc = nullptr;
  int4* tc_tiles = nullptr;
  GSTask* gs = nullptr;
  EigFTask* eigf = nullptr;
  WSDTask* wsd = nullptr;
  WSDTerm* wsd_terms = nullptr;
  VPotTask* vpot = nullptr;
  VCoord* vcoords = nullptr;
  int2* vpot_tiles = nullptr;
  PotTerm* pot_terms = nullptr;
  PotFactor* pot_factors = nullptr;
  int n_pot_terms = 0, n_modes = 0;
  int wsd_max_n = 0, wsd_max_d = 0;
  DVLTask* dvl = nullptr;
  int2* dvl_tiles = nullptr;
  EWTask* ew = nullptr;
  int2* ew_tiles = nullptr;
  int* status = nullptr;  // device status word: non-zero when a tensor-core stage gave up waiting
};
// prec 0: complex128 on the FP64 pipe; 1: double-float on the FP32 pipe
cudaError_t launch_stage(const Stage& st, const DevTables& t, double eps, int max_eig_d, int prec,
                         cudaStream_t s);
cudaError_t launch_set_identity(double2* m, int d, int prec, cudaStream_t s);
// single-op launches for the primitive C ABI calls
cudaError_t launch_single_mp(const MPTask& task, cudaStream_t s, void* scratch);
// Householder QR of node tensors, one block per task {A, R, Qs, m, n}: A (m x n)
// replaced by its thin Q, R (n x n) written, Qs (m x n) scratch
struct QRTask {
  double2* A;
  double2* R;
  double2* Qs;
  int m, n;
};
cudaError_t launch_house_qr(const void* tasks, int n_tasks, cudaStream_t s);
cudaError_t launch_single_hp(const HPTask& task, cudaStream_t s, void* scratch);
// allocation-free density inverse (scratch in a static device array)
int64_t static_eig_capacity();
cudaError_t launch_rho_inverse_static(const double2* rho, double2* rhoinv, int n_mats, int d,
                                      double eps, cudaStream_t s);
// out = x + a * y on n complex128 numbers (x may alias out)
// Outputs per thread (rows x cols, 1..4 each) of a hole-product tile of m x m
// (m <= 64): the fewest whose thread grid ceil(m/rows) x ceil(m/cols) fits
// 256 threads and 64 staged columns.
inline void hp_shape(int m, int* rows, int* cols) {
  int best = 1 << 30;
  *rows = *cols = 4;
  for (int r = 1; r <= 4; ++r)
    for (int c = 1; c <= 4; ++c) {
      const int tr = (m + r - 1) / r, tc = (m + c - 1) / c;
      if (tr * tc > 256 || tr * r > 64 || tc * c > 64) continue;
      if (r * c < best) {
        best = r * c;
        *rows = r;
        *cols = c;
      }
    }
}
// One complex128 hole product split over its reduction index (partial tiles
// in ws, at most ws_elems elements); S written in full.
cudaError_t launch_hp_split(const HPTask& task, double2* ws, int64_t ws_elems, cudaStream_t s);
// SCF Krylov helpers (complex128): out[0] = sum conj(a) b (out needs 257
// elements of workspace); out = sum_t c_t v_t
constexpr int kLinCombMax = 32;
struct LinComb {
  const double2* v[kLinCombMax];
  double2 c[kLinCombMax];
  int count;
};
cudaError_t launch_dot(const double2* a, const double2* b, int64_t n, double2* out, cudaStream_t s);
// complex128 <-> double-float copy (dir 0: to double-float)
cudaError_t launch_convert(void* dst, const void* src, int64_t n, int dir, cudaStream_t s);
cudaError_t launch_lincomb(double2* out, const LinComb& lc, int64_t n, cudaStream_t s);
cudaError_t launch_axpy(double2* out, const double2* x, double2 a, const double2* y, int64_t n,
                        cudaStream_t s);
// FP64 FMA throughput probe (TFLOP/s) on the given stream; synchronises it
cudaError_t probe_fp64_peak(cudaStream_t s, double* tflops);
// mode products on the tensor cores (qt_umma.cu, tcgen05): oz = true runs the
// double-float digit arithmetic, false split-TF32 for complex64 plans; a task
// qualifies when it is not diagonal and a_in, a_out <= 64.  A wait that runs
// out writes a non-zero code to *status.
cudaError_t launch_mp_tc(bool oz, const MPTask* tasks, const int2* tiles, int64_t first_tile, int64_t n_tiles,
                         const int* tc_tasks, int64_t first_task, int64_t n_tasks, int* status, cudaStream_t s);
constexpr int kMpOzRows = 32;  // the planner's tensor-core tiles: kMpOzSub x kMpOzRows = 128 rows (b, c)
constexpr int kMpOzSub = 4;
// bytes per task of the h operand's shared-memory image (written by the
// stage's pre-pass): 4 chunks of 16 k x 7 digits x re/im x 64 x 16 bf16, then
// 64 row exponents (int)
constexpr int64_t kMpOzImageBytes = (int64_t)4 * 7 * 2 * 64 * 16 * 2 + 64 * 4;
inline int64_t mp_oz_h_bytes() { return kMpOzImageBytes; }
// hole products on the tensor cores: items (group, range z, first chunk, end
// chunk) of one stage, a CTA takes a contiguous run of them; image units
// (group, chunk) of the pre-pass that writes A's images
cudaError_t launch_hp_tc(const HPTask* tasks, const HpTcGroup* groups, const int4* items, int64_t first_item,
                         int64_t n_items, const int2* img_units, int64_t first_unit, int64_t n_units,
                         double2* ws, int* status, cudaStream_t s);
// accumulations on the tensor cores: items (task, 128-row block, units
// before the item in the stage, 0), one unit per term; image units (task,
// term) of the pre-pass that writes alpha H_t
cudaError_t launch_acc_tc(const AccTask* tasks, const AccTerm* terms, const int4* items, int64_t first_item,
                          int64_t n_items, int64_t units, const int2* img_units, int64_t first_unit,
                          int64_t n_units, int* status, cudaStream_t s);
// weighted simultaneous diagonalisation, one warp per task (qt_wsd.cu)
// max_n / max_d bound the tasks' matrix counts and orders (shared memory)
cudaError_t launch_wsd(const WSDTask* tasks, const WSDTerm* terms, int64_t first, int64_t n, int max_n,
                       int max_d, cudaStream_t s);
cudaError_t probe_df64_peak(cudaStream_t s, double* tflops);

}  // namespace qt
