/*
 * qtgpu.h -- C ABI of the GB300 tree-tensor-network H.Psi sweep library
 * (libqtgpu.so).
 *
 * The library replaces, on one GPU, the hot path of QuTree's ML-MCTDH
 * derivative: the mode-k products, hole / dot-product contractions, the
 * bottom-up SparseMatrixTree represent sweep, the top-down mean-field sweep,
 * the density-matrix tree with its regularised inverse, and the per-node
 * sum-of-products H.Psi application (Apply / LayerDerivative / Derivative).
 *
 * Conventions (identical to QuTree's):
 *  - complex numbers are interleaved (re, im) doubles;
 *  - a node tensor of shape (d_0, ..., d_{k-1}, d_up) is column-major, the
 *    first index fastest (include/Core/Tensor_Implementation.h:154-165 of the
 *    reference); matrices are column-major, M(i,j) = m[i + j*dim1];
 *  - nodes are numbered in QuTree's bottom-up address order
 *    (src/TreeShape/Tree.cpp:92-114): children before parents, the top last;
 *  - "packed" wavefunction layout: node tensors back to back in address
 *    order, no padding.
 *
 * Every call returns a status (QT_OK on success).  The library never exits
 * the process; qt_last_error() describes the last failure of a context.
 * A call makes its context's device current while it runs and restores the
 * caller's current device before it returns.  A CUDA error that earlier work
 * of the calling thread left pending is reported (QT_ERR_CUDA, named as
 * pending in qt_last_error) rather than cleared silently.
 * Fault injection for tests: with QT_FAULT_INJECT=alloc:N in the
 * environment, the N-th device allocation of the library (counted from the
 * moment the variable took that value) fails as if the device were out of
 * memory, and the call that made it returns QT_ERR_ALLOC.
 * Calls on one context are ordered on that context's CUDA stream; a context
 * must not be used from two host threads at once.
 */
#ifndef QTGPU_H
#define QTGPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define QT_OK 0
#define QT_ERR_ARG 1     /* null pointer, bad enum, call out of order        */
#define QT_ERR_SHAPE 2   /* inconsistent tree / operator / tensor geometry   */
#define QT_ERR_ALLOC 3   /* device or host allocation failed                 */
#define QT_ERR_CUDA 4    /* a CUDA runtime call failed                       */
#define QT_ERR_STATE 5   /* call needs an earlier step (upload, prepare, ...) */
#define QT_ERR_NUMERIC 6 /* non-finite input or result                       */
#define QT_ERR_TIMEOUT 7 /* a tensor-core kernel's wait ran out (its CTAs
                            freed their resources and returned; the results
                            of that sweep are void); reported, and cleared, by
                            the next qt_sync, qt_energies or qt_dpsi_download */

/* Leaf operator kinds of the operator table. */
#define QT_OP_DENSE 0 /* p x p complex matrix, column-major                  */
#define QT_OP_DIAG 1  /* p complex numbers (operator diagonal in the DVR)    */

/* Plan flavours for qt_prepare. */
#define QT_PLAN_REFERENCE 0 /* one represent / mean-field / apply chain per SOP
                               term and node, the reference's call sequence   */
#define QT_PLAN_GROUPED 1   /* terms with identical restrictions share their
                               matrices and chains; Apply sums the mean fields
                               of terms with the same inside part first       */
#define QT_PLAN_COMPRESSED 2 /* only the sums the sweep consumes: per node one
                               block matrix of the terms inside its subtree,
                               per boundary restriction one represent matrix
                               and one summed mean field; represent chain
                               outputs stay in device memory for Apply.  No
                               per-term matrices (QT_MAT_HMAT / QT_MAT_HCON
                               downloads return QT_ERR_STATE)                */

/* Arithmetic of the sweep, OR-ed into the plan flavour of qt_prepare.
 * QT_PREC_F64: complex128 on the FP64 pipe.
 * QT_PREC_DF64: every real number carried as an unevaluated sum of two
 * floats (hi + lo, ~48-bit significand) and computed on the FP32 pipe, which
 * GB300 runs 61x faster than FP64; the density-matrix inverses stay
 * complex128 (their regularisation acts on eigenvalues down to eps).  Inputs
 * and outputs of the C ABI are complex128 in both cases. */
#define QT_PREC_F64 0x000
#define QT_PREC_DF64 0x100
/* Double-float arithmetic as QT_PREC_DF64, with the mode products (k <= 64
 * indices in and out) on the fifth-generation tensor cores (tcgen05.mma,
 * accumulators in tensor memory); hole products and last-index
 * accumulations stay on the FP32 pipe.  Every operand row is scaled by a
 * power of two and cut into seven signed digits of at most eight bits by
 * error-free splits, digit products are exact in bf16, each level of digit
 * pairs sums exactly in fp32 as far as tensor memory holds separate level
 * accumulators (all seven for outputs padded to <= 32 columns, five for 48,
 * four for 64, the last taking the remaining levels), and the levels are
 * recombined in double-float.  The error is relative to the row maxima of
 * the operands: 2^-49 of the row scale per value, plus the fp32 rounding of
 * the last level accumulator.  Parity tolerance 1e-10 per contraction and
 * projected derivative; energies agree with complex128 to ~1e-13 relative. */
#define QT_PREC_DF64_TC 0x200
/* Complex64 arithmetic: every contraction of the sweep computes in complex
 * FP32 (FP32 multiply-adds and sums, unit roundoff 2^-24) on the FP32 pipe;
 * node tensors and matrices keep the 16-byte layout of the other
 * arithmetics (their low words unused).  The density-matrix inverses stay
 * complex128 as in QT_PREC_DF64.  Error against complex128 ~1e-7 relative
 * per contraction: the mixed-precision end of the scale, with the error of
 * every result stated against the complex128 path.  Inputs and outputs of
 * the C ABI stay complex128. */
#define QT_PREC_C32 0x400
/* QT_PREC_C32 with the mode products on the tensor cores as split-TF32
 * (3 passes: hi*hi + hi*lo + lo*hi of TF32 halves, FP32 accumulation in
 * tensor memory).  Same accuracy class as QT_PREC_C32. */
#define QT_PREC_TF32X3 0x800

/* OR-ed into the plan flavour: every sweep also computes the gradient of
 * E = <Psi|H|Psi>/<Psi|Psi> with respect to every node tensor,
 * dE/dPhi_n^* (Wirtinger), assuming the orthonormal gauge QuTree keeps
 * (all non-top nodes orthonormal): (Apply(n) + Phi_n x_last Eout[n]
 * - E Phi_n x_last rho[n]) / <Psi|Psi>, with Eout[n] the mean field of the
 * terms acting only outside n.  Read it with qt_gradient_download.  No
 * counterpart in the reference (QuTree has no tree-network gradient). */
#define QT_PLAN_GRADIENT 0x1000

/* OR-ed into QT_PLAN_COMPRESSED (either arithmetic; with QT_PREC_DF64 the
 * effective Hamiltonian and the rebuilds run in double-float, the Lanczos
 * vectors and the QR in complex128): also plan the SCF / Krylov sweep of qt_scf -- the HamiltonianRepresentation(H, tree, tree,
 * tail = false) of QuTree's SCF with its correction matrices
 * (include/TreeClasses/HamiltonianRepresentation.h:19-177,
 * src/TreeClasses/HamiltonianRepresentation.cpp:117-203). */
#define QT_PLAN_SCF 0x2000

/* OR-ed into QT_PLAN_REFERENCE or QT_PLAN_GROUPED (complex128, one tree):
 * the Hamiltonian also has a potential, uploaded with qt_cdvr_upload, that
 * the sweep applies by CDVR, as QuTree does when H.hasV
 * (src/TreeClasses/HamiltonianRepresentation.cpp:30-32,
 * include/TreeClasses/HamiltonianRepresentation.h:84-86): CDVR::Update
 * (src/DVR/CDVR.cpp:150-175) inside every build and CDVR::apply
 * (src/DVR/CDVR.cpp:90-123) added to Apply at every node.  Everything runs
 * on the device inside the sweep's graph. */
#define QT_PLAN_CDVR 0x4000

/* Matrix sets for qt_matrices_download. */
#define QT_MAT_RHO 0     /* density matrices, per node, d_up x d_up          */
#define QT_MAT_RHOINV 1  /* regularised inverse density matrices             */
#define QT_MAT_HMAT 2    /* represent matrices, sparse layout                */
#define QT_MAT_HCON 3    /* mean-field (hole) matrices, sparse layout         */
#define QT_MAT_CDVR 4    /* the whole CDVR arena (grids, transformations,
                            potentials, correction tensors), complex128    */

/* qt_cdvr_upload flag: hand every hole grid its own mode's diagonal.  The
 * reference hands them out by rank among the node's active grid trees
 * (setGrids, src/DVR/TDDVR.cpp:22-30), which on upper nodes gives some hole
 * grids the diagonal of another mode's X matrix; the default reproduces it. */
#define QT_CDVR_ALIGNED_HOLE_GRIDS 1

typedef struct qt_ctx qt_ctx;

/* ---- context -------------------------------------------------------------
 * One context = one CUDA device, one stream, and the device arena of one
 * tree, one SOP operator and one wavefunction.  Replaces the reference's
 * per-call allocations and WorkMemory scratch
 * (include/TreeClasses/WorkMemory.h:9-60). */
int qt_ctx_create(qt_ctx** ctx, int device);
void qt_ctx_destroy(qt_ctx* ctx);
const char* qt_last_error(const qt_ctx* ctx);
int qt_sync(qt_ctx* ctx);
/* The context's CUDA stream (a cudaStream_t), for callers that order their
 * own work with the library's. */
int qt_get_stream(qt_ctx* ctx, void** stream);

/* ---- inputs --------------------------------------------------------------
 * Tree topology (replaces Tree / Node / TensorShape,
 * include/TreeShape/Tree.h, include/Core/TensorShape.h:5-67).
 *   order[n]     number of indices of node n (children + 1; 2 for bottom)
 *   dims[]       the node shapes back to back, last index = d_up
 *   parent[n]    parent address, -1 for the top
 *   child_idx[n] position of n among its parent's children (-1 for top)
 *   leaf_mode[n] physical mode of a bottom node, -1 for upper nodes */
int qt_tree_upload(qt_ctx* ctx, int n_nodes, const int* order, const int* dims,
                   const int* parent, const int* child_idx, const int* leaf_mode);

/* SOP operator (replaces SOPcd / MLOcd / LeafMatrix / LeafFunction,
 * include/TreeOperators/SumOfProductsOperator.h:5-135,
 * include/TreeOperators/MultiLeafOperator.h:11-196).
 *   op_kind/op_dim/op_off  leaf operator table; op_off in complex elements
 *                          into op_data
 *   coeff[2*n_terms]       complex coefficient of each term
 *   term_ptr[n_terms+1]    CSR pointer into term_mode / term_op
 *   term_mode, term_op     factor (leaf mode, operator) list of each term;
 *                          factors on the same leaf are applied in list
 *                          order (MultiLeafOperator::apply,
 *                          src/TreeOperators/MultiLeafOperator.cpp:11-37) */
int qt_sop_upload(qt_ctx* ctx, int n_ops, const int* op_kind, const int* op_dim,
                  const int64_t* op_off, const double* op_data, int n_terms,
                  const double* coeff, const int* term_ptr, const int* term_mode,
                  const int* term_op);

/* Potential of a Hamiltonian with hasV, applied by CDVR (QT_PLAN_CDVR).
 * Replaces PotentialOperator / Potential::evaluate
 * (include/TreeOperators/PotentialOperator.h:14-62,
 * include/TreeOperators/Potential.h:9-18) and the leaves' DVR grids
 * (LeafInterface::getX, include/TreeShape/LeafTypes/DVRBasis.h:27-29).
 *   leaf_dim[m], leaf_x[]   the DVR grid points of every mode m, back to back
 *   coeff[q], term_ptr[]    V(x) = sum_q coeff[q] prod x_{term_mode}^{term_power}
 *   term_mode, term_power   over the factors [term_ptr[q], term_ptr[q+1]);
 *                           a device-side polynomial stands in for the
 *                           reference's C++ potential callback (e.g.
 *                           contrib's CDVRModelV is 2f terms)
 *   flags                   QT_CDVR_ALIGNED_HOLE_GRIDS or 0 */
int qt_cdvr_upload(qt_ctx* ctx, int n_modes, const int* leaf_dim, const double* leaf_x,
                   int n_terms, const double* coeff, const int* term_ptr,
                   const int* term_mode, const int* term_power, int flags);

/* Regularisation epsilon of the inverse density matrices,
 * lambda -> 1/(lambda + eps*exp(-lambda/eps)); default 1e-10 as
 * HamiltonianRepresentation::build uses
 * (include/TreeClasses/HamiltonianRepresentation.h:72). */
int qt_set_regularization(qt_ctx* ctx, double eps);

/* Builds the sweep plan, allocates the device arena and captures the sweep
 * as a CUDA graph.  plan_flavour = QT_PLAN_* | QT_PREC_*.  Needs tree and
 * SOP.  No allocation happens afterwards. */
int qt_prepare(qt_ctx* ctx, int plan_flavour);

/* Wavefunction, packed layout (TensorTree<cd>,
 * include/TreeClasses/TensorTree.h:17-132). */
int qt_psi_upload(qt_ctx* ctx, const double* psi_host);
int qt_psi_upload_device(qt_ctx* ctx, const void* psi_dev);
int qt_psi_download(qt_ctx* ctx, double* psi_host);
int64_t qt_psi_size(const qt_ctx* ctx); /* complex elements, packed */
/* Checkpoint / resume in QuTree's TTre format ("TTre", int32 node count,
 * then per node "TENS" + "TDIM" + int32 order + int32 dims + int32 16 +
 * complex128 coefficients; TensorTree::write / read,
 * include/TreeClasses/TensorTree_Implementation.h:78-132).  Loading checks
 * every node shape against the uploaded tree (QT_ERR_SHAPE otherwise). */
int qt_psi_save(qt_ctx* ctx, const char* path);
int qt_psi_load(qt_ctx* ctx, const char* path);

/* ---- sweep ---------------------------------------------------------------
 * One H.Psi sweep = Derivative(dPsi, hRep, t, Psi, H, tree, phase)
 * (src/TreeClasses/HamiltonianRepresentation.cpp:74-81): build (density
 * matrices, regularised inverses, represent, mean fields), LayerDerivative at
 * every node, and Expectation at the top
 * (src/TreeClasses/HamiltonianRepresentation.cpp:45-51).  Asynchronous on
 * the context stream. */
int qt_derivative(qt_ctx* ctx, double phase_re, double phase_im);
int qt_dpsi_download(qt_ctx* ctx, double* dpsi_host);

/* The two halves of a sweep, for integrators that hold the matrices fixed
 * over several derivative evaluations (constant mean fields):
 * qt_build = HamiltonianRepresentation::build for the current Psi
 * (include/TreeClasses/HamiltonianRepresentation.h:62-87);
 * qt_layer_derivatives = LayerDerivative at every node with the matrices of
 * the last qt_build / qt_derivative frozen and the current Psi
 * (src/TreeClasses/HamiltonianRepresentation.cpp:53-72), into dPsi. */
int qt_build(qt_ctx* ctx);
int qt_layer_derivatives(qt_ctx* ctx, double phase_re, double phase_im);

/* Fixed-step second-order constant-mean-field propagation of the device
 * wavefunction (the scheme of CMFIntegrator::Integrate,
 * src/Applications/CMFIntegrator.cpp:25-174, without its step-size control):
 * per step, build at t, propagate the node tensors with frozen matrices to
 * t+dt/2 (n_sub RK4 substeps), build at t+dt/2, propagate Psi(t) to t+dt
 * (2*n_sub RK4 substeps) with those matrices.  phase = 1 real time,
 * phase = -i imaginary time (d Psi/dt = -i*phase*H Psi).  No
 * re-orthonormalisation: the projected equations keep the node tensors
 * orthonormal to the integrator's accuracy.  Allocates three wavefunction-
 * sized work vectors on first use.  Asynchronous. */
int qt_cmf_propagate(qt_ctx* ctx, double dt, int n_steps, int n_sub, double phase_re,
                     double phase_im);
/* SCF / Krylov sweep of QuTree's scf() (src/Applications/SCF.cpp:267-341)
 * on the wavefunction of the context (plans prepared with
 * QT_PLAN_COMPRESSED | QT_PLAN_SCF, one tree): build the tail-free matrices
 * and corrections bottom-up, then n_iter sweeps over the nodes in depth-first
 * order (top, child subtree, top, ...): at every node a Lanczos space of
 * n_krylov vectors of the effective Hamiltonian (SCF.cpp:36-84,138-195),
 * imaginary-time propagation by beta for the first n_itp sweeps
 * (SCF.cpp:197-222) or the lowest Ritz vector after them, isometrisation
 * toward the next node (Cholesky-QR twice; Householder QR when the Gram
 * matrix is near singular) with R multiplied into the next node, and the
 * edge-local rebuild (buildUp / buildDown).  ritz (may be NULL) receives the
 * lowest Ritz value of every Krylov solve, n_iter * (2 * nodes - 1) of them;
 * ritz_count their number.  The optimised wavefunction stays in the context
 * (qt_psi_download).  1 <= n_krylov <= 30.  When a Lanczos residual falls
 * below 1e-12 of the Lanczos matrix norm the space is invariant and ends
 * there (the reference divides by the vanishing norm, SCF.cpp:171-173, and
 * continues on rounding noise).  Synchronises. */
int qt_scf(qt_ctx* ctx, int n_iter, int n_krylov, int n_itp, double beta, double* ritz,
           int64_t ritz_capacity, int64_t* ritz_count);
/* Energy gradient of the last sweep (plans prepared with QT_PLAN_GRADIENT),
 * packed layout like the wavefunction.  Synchronises. */
int qt_gradient_download(qt_ctx* ctx, double* grad_host);
int qt_dpsi_device(qt_ctx* ctx, const void** dpsi_dev);
/* out[4] = { Re h00, Im h00, Re S00, Im S00 }, h00 = <Phi_top|H Phi_top>,
 * S00 = <Phi_top|Phi_top>; E = Re h00 / Re S00. Synchronises.  For a forest,
 * the first tree. */
int qt_energy(qt_ctx* ctx, double* out4);

/* Forests.  The tree descriptor may hold several independent trees: every
 * node with parent -1 closes one tree, whose nodes precede it.  Leaf modes
 * are numbered across the whole forest and every SOP term acts on the leaves
 * of one tree only (terms on several trees fail in qt_prepare with
 * QT_ERR_SHAPE).  All trees advance together: each level's chains of every
 * tree share one launch, one CUDA graph per sweep.  No counterpart in the
 * reference, which handles one tree per HamiltonianRepresentation. */
int qt_tree_count(const qt_ctx* ctx);
/* out[4*t .. 4*t+3] = { Re h00, Im h00, Re S00, Im S00 } of tree t (roots in
 * ascending address order), for t < n_trees. Synchronises. */
int qt_energies(qt_ctx* ctx, double* out, int n_trees);

/* Matrices of the last sweep or qt_build (QT_ERR_STATE before either).
 * Sparse layout (QT_MAT_HMAT / QT_MAT_HCON):
 * for each term, for each node on its leaf-to-root paths (SparseTree with
 * tail, src/TreeClasses/SparseTree.cpp:33-89) in address order, a d_up x d_up
 * matrix.  Dense layout (QT_MAT_RHO / QT_MAT_RHOINV): per node in address
 * order.  The top node's represent matrix is zero, as in the reference. */
int64_t qt_matrices_size(const qt_ctx* ctx, int which);
int qt_matrices_download(qt_ctx* ctx, int which, double* host);

/* Plan statistics: out[0] reference-algorithm flops per sweep, out[1]
 * executed flops per sweep, out[2] kernel launches per sweep, out[3] device
 * arena bytes, out[4] scratch bytes, out[5] represent chains, out[6]
 * mean-field chains, out[7] apply chains. */
int qt_plan_stats(const qt_ctx* ctx, double* out8);

/* ---- profiling ------------------------------------------------------------
 * The prepared sweep is a fixed sequence of batched kernel launches
 * ("stages").  These calls expose it for per-kernel timing: a caller can
 * launch stage i alone on the context stream (outside the graph, with the
 * same arguments the graph uses) and bracket it with its own CUDA events.
 * kind: 0 mode products, 1 hole products, 2 last-mode accumulations,
 * 3 mean-field sums, 4 density inverses, 5 projectors. */
int qt_stage_count(const qt_ctx* ctx);
int qt_stage_info(const qt_ctx* ctx, int stage, int* kind, int64_t* tiles, double* flops,
                  double* bytes);
int qt_stage_launch(qt_ctx* ctx, int stage);
/* Peak FP64 FMA throughput of the device (TFLOP/s), measured with a dependent-
 * free FMA loop of the library's own; the roofline denominator of the
 * complex128 kernels. */
int qt_probe_fp64_peak(qt_ctx* ctx, double* tflops);
/* Ceiling of the double-float arithmetic (TFLOP/s, complex128-equivalent:
 * 8 flops per complex multiply-add): the kernels' double-float complex
 * multiply-add and renormalisation on register accumulators, no memory
 * traffic; the roofline denominator of the QT_PREC_DF64 kernels.  No
 * reference counterpart (diagnostic). */
int qt_probe_df64_peak(qt_ctx* ctx, double* tflops);

/* ---- primitives on device pointers ---------------------------------------
 * Mode-k product, the reference's matvec_ / matrixTensor
 * (include/Core/Tensor_Implementation.h:450-461,553-577; src/Core/LA_lib.f:34-81):
 *   C[b, a', c] (+)= sum_a h(a', a) B[b, a, c],
 *   h is activeC x activeB, column-major; add != 0 accumulates. */
int qt_mode_product(qt_ctx* ctx, void* C, const void* h, const void* B, int64_t before,
                    int64_t activeB, int64_t activeC, int64_t after, int add);
/* Hole product, the reference's rhomat_ / contraction
 * (include/Core/Tensor_Implementation.h:481-531; src/Core/LA_lib.f:718-762):
 *   S(a, a') = sum_{b,c} conj(A[b, a, c]) B[b, a', c]. */
int qt_hole_product(qt_ctx* ctx, void* S, const void* A, const void* B, int64_t before,
                    int64_t activeA, int64_t activeB, int64_t after);
/* Last-mode product multStateAB (include/Core/Tensor_Implementation.h:732-760):
 *   C[i, m] (+)= sum_n A(m, n) B[i, n], B is (lastBefore x active). */
int qt_last_mode_product(qt_ctx* ctx, void* C, const void* A, const void* B,
                         int64_t last_before, int64_t active, int add);

/* Regularised inverses rhoinv[b] = U diag(1/(w + eps*exp(-w/eps))) U^dagger
 * of n_mats Hermitian d x d matrices rho[b] (column-major, back to back) that
 * already live on the device, without any device allocation.  The ranges
 * rho[0 .. n_mats*d*d) and rhoinv[0 .. n_mats*d*d) must not overlap
 * (QT_ERR_ARG otherwise).
 *
 * This entry point has no counterpart in the reference.  It exists for
 * callers that cannot call cudaMalloc: code that runs while a CUDA stream is
 * being captured into a graph (allocation calls are not allowed there),
 * latency-critical loops that cannot afford the device-wide synchronisation
 * of cudaFree, and hosts whose device memory belongs to a pooling allocator
 * that forbids side allocations.  The caller passes inputs and outputs; the
 * Jacobi workspace is a static device array of 8 MiB owned by the library,
 * held on every GPU that loads it until the process exits.
 *   - n_mats * d * d must be <= 524288 (complex elements) and d <= 112;
 *     larger requests fail with QT_ERR_SHAPE and launch nothing.
 *   - The first call on a device looks up the array's device address
 *     (cudaGetSymbolAddress), and so does the first call after the
 *     device's context was replaced (cudaDeviceReset); make those calls
 *     before any stream capture starts (inside a capture they fail with
 *     QT_ERR_CUDA rather than use a stale address).
 *   - All calls share the workspace: calls that overlap on the GPU (other
 *     streams, contexts or threads) race and must be serialised by the
 *     caller.  The workspace needs no clearing between calls.
 * Asynchronous on the context stream. */
int qt_rho_inverse_noalloc(qt_ctx* ctx, void* rhoinv, const void* rho, int n_mats, int d,
                           double eps);

/* Lower bounds of the shapes the next qt_prepare puts on the tensor cores
 * (QT_PREC_DF64_TC; QT_PREC_TF32X3 uses the mode-product bound): mode
 * products with mp_min <= a_in, a_out <= 64, hole products with
 * hp_min <= a <= 64, accumulations with acc_min <= d <= 64; 65 keeps a kind
 * on the FP32 pipe.  Defaults 32, 32, 32 (measured on GB300); the autotuner
 * (qutree_gb300/autotune.py) times probe problems per size on the device
 * and caches the bounds per device.  QT_ERR_ARG outside 1..65. */
int qt_set_tc_thresholds(qt_ctx* ctx, int mp_min, int hp_min, int acc_min);

/* qrOrthogonal (include/TreeClasses/TensorTree_Implementation.h:173-187) on
 * the uploaded wavefunction, in place on the device: bottom-up, every
 * non-top node tensor, as a (lastBefore x d_up) matrix, is replaced by the
 * thin Q of its Householder QR (qr, include/Core/Matrix_Implementation.h:
 * 795-806: reflectors mapping each column to -e^{i arg x_0} |x| e_1, as
 * Eigen's HouseholderQR) and R = Q^H Phi is multiplied into the parent along
 * the node's child index (matrixTensor).  Complex128 on the FP64 pipe, one
 * block per node; the nodes of one height run together.  Uses the
 * context's chain scratch (QT_ERR_ALLOC when a height's Q and R do not fit).
 * QT_ERR_STATE without a prepared context and an uploaded wavefunction. */
int qt_qr_orthogonal(qt_ctx* ctx);

/* Device memory helpers for callers without their own allocator. */
int qt_dev_alloc(qt_ctx* ctx, int64_t bytes, void** ptr);
int qt_dev_free(qt_ctx* ctx, void* ptr);
int qt_memcpy_h2d(qt_ctx* ctx, void* dst, const void* src, int64_t bytes);
int qt_memcpy_d2h(qt_ctx* ctx, void* dst, const void* src, int64_t bytes);

/* Number of the library's own kernel launches enqueued since the context was
 * created (graph launches count their kernels). */
int64_t qt_launch_count(const qt_ctx* ctx);

#ifdef __cplusplus
}
#endif
#endif /* QTGPU_H */
