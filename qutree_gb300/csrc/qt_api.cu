// qt_api.cu -- the extern "C" entry points of libqtgpu (include/qtgpu.h).
//
// A context owns one CUDA stream and one device arena: the wavefunction, its
// H.Psi and derivative (packed TensorTree layout), all d x d matrices of the
// sweep (density, inverse density, represent, mean-field, grouped mean-field
// and projector matrices), the leaf operator table, the chain scratch and the
// task tables of the plan.  qt_prepare allocates all of it once and captures
// the whole sweep as one CUDA graph; qt_derivative only launches that graph.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/qtgpu.h"
#include "qt_internal.h"

using qt::Plan;
using qt::Ref;

struct qt_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  std::string err;
  bool have_tree = false, have_sop = false, prepared = false, have_psi = false, swept = false;
  bool built = false;  // matrices of the current plan computed (qt_build / qt_derivative)
  std::vector<qt::NodeGeo> nodes;
  qt::OpTable ops;
  qt::SopDesc sop;
  qt::CdvrDesc cdvr;  // potential of a Hamiltonian with hasV (qt_cdvr_upload)
  qt::TcTune tune;     // tensor-core bounds for the next qt_prepare (qt_set_tc_thresholds)
  bool have_cdvr = false;
  double eps = 1e-10;
  Plan plan;
  double2* buf[qt::B_NBUF] = {nullptr};
  int64_t buf_elems[qt::B_NBUF] = {0};
  void* tables_mem = nullptr;
  qt::DevTables tables;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaGraphExec_t exec_build = nullptr;  // stages [0, apply_begin)
  cudaGraphExec_t exec_apply = nullptr;  // [psi-in conversion] + stages [apply_begin, end)
  double2* cmf_buf[3] = {nullptr, nullptr, nullptr};  // CMF work vectors, allocated on first use
  int64_t launches = 0;
  int prec = 0;
  std::vector<double> ops_df;  // double-float operator table staging (prec 1)
};

namespace {

thread_local std::string g_noctx_err;

int fail(qt_ctx* c, int code, const std::string& msg) {
  if (c)
    c->err = msg;
  else
    g_noctx_err = msg;
  return code;
}

int cuda_fail(qt_ctx* c, cudaError_t e, const char* where) {
  return fail(c, QT_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

#define QT_CUDA(c, call)                                  \
  do {                                                    \
    cudaError_t e_ = (call);                              \
    if (e_ != cudaSuccess) return cuda_fail(c, e_, #call); \
  } while (0)

// Makes the context's device current for the duration of one entry point and
// restores the caller's current device on return, so that a host application
// driving several GPUs keeps its own device selection.  It also reports a
// CUDA error left pending by earlier, unrelated work of the calling thread
// instead of silently clearing it.
struct DevScope {
  int prev = -1;
  cudaError_t err = cudaSuccess;
  bool pending = false;
  explicit DevScope(int device) {
    err = cudaGetDevice(&prev);
    if (err != cudaSuccess) {
      prev = -1;
      return;
    }
    if (prev != device) err = cudaSetDevice(device);
    if (err != cudaSuccess) return;
    err = cudaGetLastError();
    pending = err != cudaSuccess;
  }
  ~DevScope() {
    int cur = -1;
    if (prev >= 0 && cudaGetDevice(&cur) == cudaSuccess && cur != prev) cudaSetDevice(prev);
  }
};

#define QT_DEVICE(c)                                                                                       \
  DevScope dev_scope_((c)->device);                                                                        \
  do {                                                                                                     \
    if (dev_scope_.err != cudaSuccess)                                                                     \
      return fail(c, QT_ERR_CUDA,                                                                          \
                  std::string(__func__) +                                                                  \
                      (dev_scope_.pending ? ": a CUDA error was pending from earlier work of this thread: " \
                                          : ": cannot make the context's device current: ") +              \
                      cudaGetErrorString(dev_scope_.err));                                                 \
  } while (0)

// Every device allocation of the library goes through dev_malloc, so that a
// test can make a chosen one fail without exhausting the GPU:
// QT_FAULT_INJECT=alloc:N makes the N-th allocation counted from the moment
// the variable took its current value fail with cudaErrorMemoryAllocation.
cudaError_t dev_malloc(void** p, size_t bytes) {
  static std::mutex mu;
  static std::string spec;
  static long count = 0;
  long nth = 0;
  {
    std::lock_guard<std::mutex> lock(mu);
    const char* v = std::getenv("QT_FAULT_INJECT");
    const std::string cur = v ? v : "";
    if (cur != spec) {
      spec = cur;
      count = 0;
    }
    if (spec.compare(0, 6, "alloc:") == 0) {
      nth = std::atol(spec.c_str() + 6);
      ++count;
    }
  }
  if (nth > 0 && count == nth) {
    *p = nullptr;
    return cudaErrorMemoryAllocation;
  }
  return cudaMalloc(p, bytes);
}

void release_arena(qt_ctx* c) {
  if (c->exec) cudaGraphExecDestroy(c->exec);
  if (c->graph) cudaGraphDestroy(c->graph);
  if (c->exec_build) cudaGraphExecDestroy(c->exec_build);
  if (c->exec_apply) cudaGraphExecDestroy(c->exec_apply);
  for (auto& b : c->cmf_buf) {
    if (b) cudaFree(b);
    b = nullptr;
  }
  c->exec = nullptr;
  c->graph = nullptr;
  c->exec_build = nullptr;
  c->exec_apply = nullptr;
  // B_PSI64 / B_DPSI64 alias B_PSI / B_DPSI in complex128 plans: free once
  if (c->buf[qt::B_PSI64] == c->buf[qt::B_PSI]) c->buf[qt::B_PSI64] = nullptr;
  if (c->buf[qt::B_DPSI64] == c->buf[qt::B_DPSI]) c->buf[qt::B_DPSI64] = nullptr;
  if (c->buf[qt::B_GRAD64] == c->buf[qt::B_GRAD]) c->buf[qt::B_GRAD64] = nullptr;
  for (int i = 0; i < qt::B_NBUF; ++i) {
    if (c->buf[i]) cudaFree(c->buf[i]);
    c->buf[i] = nullptr;
    c->buf_elems[i] = 0;
  }
  if (c->tables_mem) cudaFree(c->tables_mem);
  c->tables_mem = nullptr;
  c->tables = qt::DevTables();
  c->prepared = false;
  c->have_psi = false;
  c->swept = false;
  c->built = false;
}

const double2* ptr_of(const qt_ctx* c, const Ref& r) {
  if (r.buf < 0) return nullptr;
  return c->buf[r.buf] + r.off;
}
double2* mptr_of(const qt_ctx* c, const Ref& r) {
  if (r.buf < 0) return nullptr;
  return c->buf[r.buf] + r.off;
}

template <typename T>
void put(std::vector<char>& blob, std::vector<int64_t>& offs, const std::vector<T>& v) {
  size_t o = (blob.size() + 255) / 256 * 256;
  blob.resize(o + v.size() * sizeof(T));
  if (!v.empty()) std::memcpy(blob.data() + o, v.data(), v.size() * sizeof(T));
  offs.push_back((int64_t)o);
}

bool finite_all(const double* p, int64_t n) {
  for (int64_t i = 0; i < n; ++i)
    if (!std::isfinite(p[i])) return false;
  return true;
}

}  // namespace

extern "C" {

int qt_ctx_create(qt_ctx** out, int device) {
  if (!out) return fail(nullptr, QT_ERR_ARG, "qt_ctx_create: null output pointer");
  *out = nullptr;
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess) return fail(nullptr, QT_ERR_CUDA, std::string("cudaGetDeviceCount: ") + cudaGetErrorString(e));
  if (device < 0 || device >= n) return fail(nullptr, QT_ERR_ARG, "qt_ctx_create: no such device");
  qt_ctx* c = new (std::nothrow) qt_ctx();
  if (!c) return fail(nullptr, QT_ERR_ALLOC, "qt_ctx_create: out of host memory");
  c->device = device;
  DevScope scope(device);
  if (scope.err != cudaSuccess) {
    delete c;
    return fail(nullptr, QT_ERR_CUDA,
                std::string("qt_ctx_create: ") +
                    (scope.pending ? "a CUDA error was pending from earlier work of this thread: " : "") +
                    cudaGetErrorString(scope.err));
  }
  e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    delete c;
    return fail(nullptr, QT_ERR_CUDA, std::string("qt_ctx_create: ") + cudaGetErrorString(e));
  }
  *out = c;
  return QT_OK;
}

void qt_ctx_destroy(qt_ctx* c) {
  if (!c) return;
  DevScope scope(c->device);
  if (c->stream) cudaStreamSynchronize(c->stream);
  release_arena(c);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
}

const char* qt_last_error(const qt_ctx* c) { return c ? c->err.c_str() : g_noctx_err.c_str(); }

namespace {
// the status word the tensor-core kernels set when a wait runs out (read
// after the stream synchronised; cleared once reported)
int check_status(qt_ctx* c) {
  if (!c->prepared || !c->tables.status) return QT_OK;
  int st = 0;
  QT_CUDA(c, cudaMemcpyAsync(&st, c->tables.status, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  QT_CUDA(c, cudaStreamSynchronize(c->stream));
  if (st == 0) return QT_OK;
  QT_CUDA(c, cudaMemsetAsync(c->tables.status, 0, sizeof(int), c->stream));
  return fail(c, QT_ERR_TIMEOUT, "a tensor-core kernel gave up waiting (code " + std::to_string(st) +
                                     "); the results of that sweep are void");
}
}  // namespace

int qt_sync(qt_ctx* c) {
  if (!c) return fail(c, QT_ERR_ARG, "null context");
  QT_DEVICE(c);
  QT_CUDA(c, cudaStreamSynchronize(c->stream));
  return check_status(c);
}

int qt_get_stream(qt_ctx* c, void** s) {
  if (!c || !s) return fail(c, QT_ERR_ARG, "null argument");
  *s = (void*)c->stream;
  return QT_OK;
}

int qt_tree_upload(qt_ctx* c, int n_nodes, const int* order, const int* dims, const int* parent,
                   const int* child_idx, const int* leaf_mode) {
  if (!c) return fail(c, QT_ERR_ARG, "null context");
  QT_DEVICE(c);
  if (n_nodes <= 0 || !order || !dims || !parent || !child_idx || !leaf_mode)
    return fail(c, QT_ERR_ARG, "qt_tree_upload: null or empty descriptor");
  release_arena(c);
  std::vector<qt::NodeGeo> nodes(n_nodes);
  int p = 0;
  for (int i = 0; i < n_nodes; ++i) {
    if (order[i] < 2 || order[i] > 8) return fail(c, QT_ERR_SHAPE, "qt_tree_upload: node order must be 2..8");
    for (int k = 0; k < order[i]; ++k) nodes[i].shape.push_back(dims[p + k]);
    p += order[i];
    nodes[i].parent = parent[i];
    nodes[i].child_idx = child_idx[i];
    nodes[i].leaf_mode = leaf_mode[i];
    if (parent[i] >= n_nodes || (parent[i] >= 0 && child_idx[i] < 0))
      return fail(c, QT_ERR_SHAPE, "qt_tree_upload: bad parent / child index");
  }
  c->nodes = nodes;
  c->have_tree = true;
  return QT_OK;
}

int qt_sop_upload(qt_ctx* c, int n_ops, const int* op_kind, const int* op_dim, const int64_t* op_off,
                  const double* op_data, int n_terms, const double* coeff, const int* term_ptr,
                  const int* term_mode, const int* term_op) {
  if (!c) return fail(c, QT_ERR_ARG, "null context");
  QT_DEVICE(c);
  if (n_ops <= 0 || n_terms <= 0 || !op_kind || !op_dim || !op_off || !op_data || !coeff ||
      !term_ptr || !term_mode || !term_op)
    return fail(c, QT_ERR_ARG, "qt_sop_upload: null or empty descriptor");
  release_arena(c);
  qt::OpTable ops;
  int64_t total = 0;
  for (int i = 0; i < n_ops; ++i) {
    if (op_kind[i] != QT_OP_DENSE && op_kind[i] != QT_OP_DIAG)
      return fail(c, QT_ERR_ARG, "qt_sop_upload: unknown operator kind");
    if (op_dim[i] <= 0 || op_off[i] < 0) return fail(c, QT_ERR_SHAPE, "qt_sop_upload: bad operator dim/offset");
    int64_t n = op_kind[i] == QT_OP_DENSE ? (int64_t)op_dim[i] * op_dim[i] : op_dim[i];
    total = std::max(total, op_off[i] + n);
  }
  // repack each operator contiguously (16-element aligned) in the device table
  int64_t cur = 0;
  for (int i = 0; i < n_ops; ++i) {
    int64_t n = op_kind[i] == QT_OP_DENSE ? (int64_t)op_dim[i] * op_dim[i] : op_dim[i];
    ops.kind.push_back(op_kind[i]);
    ops.dim.push_back(op_dim[i]);
    ops.off.push_back(cur);
    ops.data.resize(2 * (cur + n), 0.0);
    std::memcpy(ops.data.data() + 2 * cur, op_data + 2 * op_off[i], sizeof(double) * 2 * n);
    cur = (cur + n + 15) / 16 * 16;
  }
  ops.data.resize(2 * std::max<int64_t>(cur, 16), 0.0);
  if (!finite_all(ops.data.data(), (int64_t)ops.data.size()))
    return fail(c, QT_ERR_NUMERIC, "qt_sop_upload: non-finite operator entry");
  qt::SopDesc s;
  s.n_terms = n_terms;
  for (int l = 0; l < n_terms; ++l) {
    if (!std::isfinite(coeff[2 * l]) || !std::isfinite(coeff[2 * l + 1]))
      return fail(c, QT_ERR_NUMERIC, "qt_sop_upload: non-finite coefficient");
    s.coeff.push_back(make_double2(coeff[2 * l], coeff[2 * l + 1]));
  }
  s.ptr.assign(term_ptr, term_ptr + n_terms + 1);
  if (s.ptr[0] != 0) return fail(c, QT_ERR_ARG, "qt_sop_upload: term_ptr[0] must be 0");
  for (int l = 0; l < n_terms; ++l)
    if (s.ptr[l + 1] < s.ptr[l]) return fail(c, QT_ERR_ARG, "qt_sop_upload: term_ptr not monotone");
  s.mode.assign(term_mode, term_mode + s.ptr[n_terms]);
  s.op.assign(term_op, term_op + s.ptr[n_terms]);
  c->ops = ops;
  c->sop = s;
  c->have_sop = true;
  return QT_OK;
}

int qt_cdvr_upload(qt_ctx* c, int n_modes, const int* leaf_dim, const double* leaf_x, int n_terms,
                   const double* coeff, const int* term_ptr, const int* term_mode, const int* term_power,
                   int flags) {
  if (!c || !leaf_dim || !leaf_x || (n_terms > 0 && (!coeff || !term_ptr || !term_mode || !term_power)))
    return fail(c, QT_ERR_ARG, "null argument");
  QT_DEVICE(c);
  if (n_modes < 2 || n_terms < 0) return fail(c, QT_ERR_ARG, "qt_cdvr_upload: bad counts");
  qt::CdvrDesc d;
  int64_t off = 0;
  for (int m = 0; m < n_modes; ++m) {
    if (leaf_dim[m] < 1) return fail(c, QT_ERR_SHAPE, "qt_cdvr_upload: empty leaf grid");
    d.leaf_x.emplace_back(leaf_x + off, leaf_x + off + leaf_dim[m]);
    off += leaf_dim[m];
    if (!finite_all(d.leaf_x.back().data(), leaf_dim[m]))
      return fail(c, QT_ERR_NUMERIC, "qt_cdvr_upload: non-finite grid point");
  }
  if (n_terms > 0 && term_ptr[0] != 0) return fail(c, QT_ERR_ARG, "qt_cdvr_upload: term_ptr[0] != 0");
  for (int q = 0; q < n_terms; ++q) {
    if (term_ptr[q + 1] < term_ptr[q]) return fail(c, QT_ERR_ARG, "qt_cdvr_upload: term_ptr not ascending");
    d.coeff.push_back(coeff[q]);
  }
  if (!finite_all(d.coeff.data(), (int64_t)d.coeff.size()))
    return fail(c, QT_ERR_NUMERIC, "qt_cdvr_upload: non-finite coefficient");
  d.ptr.assign(term_ptr, term_ptr + (n_terms > 0 ? n_terms + 1 : 0));
  if (n_terms == 0) d.ptr.push_back(0);
  const int nf = n_terms > 0 ? term_ptr[n_terms] : 0;
  for (int q = 0; q < nf; ++q) {
    if (term_mode[q] < 0 || term_mode[q] >= n_modes) return fail(c, QT_ERR_ARG, "qt_cdvr_upload: mode out of range");
    if (term_power[q] < 0 || term_power[q] > 64) return fail(c, QT_ERR_ARG, "qt_cdvr_upload: power out of range");
    d.mode.push_back(term_mode[q]);
    d.power.push_back(term_power[q]);
  }
  d.aligned = (flags & QT_CDVR_ALIGNED_HOLE_GRIDS) != 0;
  c->cdvr = std::move(d);
  c->have_cdvr = true;
  return QT_OK;
}

int qt_set_tc_thresholds(qt_ctx* c, int mp_min, int hp_min, int acc_min) {
  if (!c) return fail(c, QT_ERR_ARG, "null context");
  for (int v : {mp_min, hp_min, acc_min})
    if (v < 1 || v > 65) return fail(c, QT_ERR_ARG, "qt_set_tc_thresholds: bounds must lie in 1..65");
  c->tune.mp = mp_min;
  c->tune.hp = hp_min;
  c->tune.acc = acc_min;
  return QT_OK;
}

int qt_set_regularization(qt_ctx* c, double eps) {
  if (!c) return fail(c, QT_ERR_ARG, "null context");
  if (!(eps > 0) || !std::isfinite(eps)) return fail(c, QT_ERR_ARG, "eps must be positive and finite");
  if (c->prepared) return fail(c, QT_ERR_STATE, "set the regularisation before qt_prepare");
  c->eps = eps;
  return QT_OK;
}

int qt_prepare(qt_ctx* c, int flavour) {
  if (!c) return fail(c, QT_ERR_ARG, "null context");
  if (!c->have_tree || !c->have_sop) return fail(c, QT_ERR_STATE, "qt_prepare needs tree and SOP");
  const int prec_bits = flavour & (QT_PREC_DF64 | QT_PREC_DF64_TC | QT_PREC_C32 | QT_PREC_TF32X3);
  if (prec_bits & (prec_bits - 1)) return fail(c, QT_ERR_ARG, "qt_prepare: more than one QT_PREC_* bit");
  const bool tensor_mp = (prec_bits & (QT_PREC_DF64_TC | QT_PREC_TF32X3)) != 0;
  // storage / arithmetic: 0 complex128, 1 double-float, 2 complex64 arithmetic
  const int prec = (prec_bits & (QT_PREC_DF64 | QT_PREC_DF64_TC)) ? 1 : (prec_bits ? 2 : 0);
  const bool grad = (flavour & QT_PLAN_GRADIENT) != 0;
  const bool scf = (flavour & QT_PLAN_SCF) != 0;
  const bool cdvr = (flavour & QT_PLAN_CDVR) != 0;
  flavour &= ~(prec_bits | QT_PLAN_GRADIENT | QT_PLAN_SCF | QT_PLAN_CDVR);
  if (cdvr && !c->have_cdvr) return fail(c, QT_ERR_STATE, "QT_PLAN_CDVR needs qt_cdvr_upload first");
  if (flavour != QT_PLAN_REFERENCE && flavour != QT_PLAN_GROUPED && flavour != QT_PLAN_COMPRESSED)
    return fail(c, QT_ERR_ARG, "unknown plan flavour");
  QT_DEVICE(c);
  release_arena(c);
  int64_t budget = (int64_t)1 << 28;  // scratch elements (4 GiB)
  if (const char* s = std::getenv("QT_SCRATCH_MIB")) {
    long v = std::atol(s);
    if (v > 0) budget = (int64_t)v * (1 << 20) / 16;
  }
  std::string msg = qt::build_plan(c->plan, c->nodes, c->ops, c->sop,
                                   flavour | (scf ? 0x2000 : 0) | (tensor_mp ? 0x8000 : 0), prec, budget, grad,
                                   cdvr ? &c->cdvr : nullptr, c->tune);
  if (!msg.empty()) return fail(c, QT_ERR_SHAPE, "qt_prepare: " + msg);
  Plan& P = c->plan;
  c->buf_elems[qt::B_PSI] = P.psi_arena;
  c->buf_elems[qt::B_HPHI] = P.psi_arena;
  c->buf_elems[qt::B_DPSI] = P.psi_arena;
  c->buf_elems[qt::B_MATS] = P.mats_size;
  c->buf_elems[qt::B_OPS] = (int64_t)c->ops.data.size() / 2;
  c->buf_elems[qt::B_SCR] = std::max<int64_t>(P.scratch_size, 16);
  c->buf_elems[qt::B_PARAM] = 16;
  c->buf_elems[qt::B_PSI64] = prec >= 1 ? P.psi_arena : 0;
  c->buf_elems[qt::B_DPSI64] = prec >= 1 ? P.psi_arena : 0;
  c->buf_elems[qt::B_GRAD] = grad ? P.psi_arena : 0;
  c->buf_elems[qt::B_GRAD64] = (grad && prec >= 1) ? P.psi_arena : 0;
  c->buf_elems[qt::B_KEEP] = P.keep_size;
  c->buf_elems[qt::B_HPW] = P.hpw_size;
  c->buf_elems[qt::B_KRY] = P.kry_size;
  c->buf_elems[qt::B_CDVR] = P.cdvr ? P.cdvr_size : 0;
  c->buf_elems[qt::B_OZ] = (P.oz_bytes + 15) / 16;
  int64_t arena = 0;
  for (int i = 0; i < qt::B_NBUF; ++i) {
    if ((i == qt::B_PSI64 || i == qt::B_DPSI64 || i == qt::B_GRAD64) && prec == 0) continue;  // aliases
    if ((i == qt::B_GRAD || i == qt::B_GRAD64) && !grad) continue;
    int64_t n = std::max<int64_t>(c->buf_elems[i], 16);
    cudaError_t e = dev_malloc((void**)&c->buf[i], n * sizeof(double2));
    if (e != cudaSuccess) {
      release_arena(c);
      return fail(c, QT_ERR_ALLOC, std::string("qt_prepare: device allocation failed: ") + cudaGetErrorString(e));
    }
    arena += n * 16;
  }
  if (prec == 0) {
    c->buf[qt::B_PSI64] = c->buf[qt::B_PSI];
    c->buf[qt::B_DPSI64] = c->buf[qt::B_DPSI];
    c->buf[qt::B_GRAD64] = c->buf[qt::B_GRAD];
  }
  c->prec = prec;
  QT_CUDA(c, cudaMemsetAsync(c->buf[qt::B_MATS], 0, c->buf_elems[qt::B_MATS] * 16, c->stream));
  QT_CUDA(c, cudaMemsetAsync(c->buf[qt::B_HPHI], 0, c->buf_elems[qt::B_HPHI] * 16, c->stream));
  QT_CUDA(c, cudaMemsetAsync(c->buf[qt::B_DPSI], 0, c->buf_elems[qt::B_DPSI] * 16, c->stream));
  QT_CUDA(c, cudaMemsetAsync(c->buf[qt::B_PARAM], 0, c->buf_elems[qt::B_PARAM] * 16, c->stream));
  if (prec >= 1) {
    // operator table as double-float pairs (hi, lo) per real number
    c->ops_df.resize(c->ops.data.size());
    float* f = (float*)c->ops_df.data();
    for (size_t i = 0; i < c->ops.data.size(); ++i) {
      const double x = c->ops.data[i];
      const float h = (float)x;
      f[2 * i] = h;
      f[2 * i + 1] = (float)(x - (double)h);
    }
    QT_CUDA(c, cudaMemcpyAsync(c->buf[qt::B_OPS], c->ops_df.data(), c->ops_df.size() * sizeof(double),
                               cudaMemcpyHostToDevice, c->stream));
  } else {
    QT_CUDA(c, cudaMemcpyAsync(c->buf[qt::B_OPS], c->ops.data.data(), c->ops.data.size() * sizeof(double),
                               cudaMemcpyHostToDevice, c->stream));
  }
  // bind the symbolic tables to device pointers
  std::vector<qt::MPTask> mp;
  for (auto& s : P.mp) {
    qt::MPTask t;
    t.in = ptr_of(c, s.in);
    t.out = mptr_of(c, s.out);
    t.h = ptr_of(c, s.h);
    t.alpha = s.alpha;
    t.before = s.before;
    t.a_in = s.a_in;
    t.a_out = s.a_out;
    t.after = s.after;
    t.diag = s.diag;
    t.add = 0;
    t.oz_h = s.oz_h >= 0 ? (void*)((char*)c->buf[qt::B_OZ] + s.oz_h) : nullptr;
    mp.push_back(t);
  }
  std::vector<qt::HPTask> hp;
  for (auto& s : P.hp) {
    qt::HPTask t;
    t.A = ptr_of(c, s.A);
    t.B = ptr_of(c, s.B);
    t.S = mptr_of(c, s.S);
    t.before = s.before;
    t.a = s.a;
    t.after = s.after;
    t.aB = 0;
    t.splits = s.splits;
    t.kchunk = s.kchunk;
    t.ws = s.ws;
    t.rows = s.rows;
    t.cols = s.cols;
    hp.push_back(t);
  }
  std::vector<qt::HpTcGroup> hp_tc;
  for (auto& s : P.hp_tc_groups) {
    qt::HpTcGroup g;
    g.A = ptr_of(c, s.A);
    g.img = (unsigned char*)c->buf[qt::B_OZ] + s.img;
    g.ex = (unsigned char*)c->buf[qt::B_OZ] + s.ex;
    g.before = s.before;
    g.a = s.a;
    g.after = s.after;
    g.ap = (s.a + 7) & ~7;
    g.n = s.n;
    g.nchunks = s.nchunks;
    for (int m = 0; m < qt::kHpTcMembers; ++m) g.member[m] = s.member[m];
    hp_tc.push_back(g);
  }
  std::vector<qt::AccTask> acc;
  for (auto& s : P.acc) {
    qt::AccTask t;
    t.out = mptr_of(c, s.out);
    t.alpha_ptr = s.alpha_ref.buf >= 0 ? ptr_of(c, s.alpha_ref) : (s.alpha_param ? c->buf[qt::B_PARAM] : nullptr);
    t.alpha = s.alpha;
    t.rows = s.rows;
    t.d = s.d;
    t.first = s.first;
    t.count = s.count;
    t.add = s.add;
    t.pad = 0;
    t.tc_img = s.tc_img >= 0 ? (void*)((char*)c->buf[qt::B_OZ] + s.tc_img) : nullptr;
    acc.push_back(t);
  }
  std::vector<qt::AccTerm> acc_terms;
  for (auto& s : P.acc_terms) acc_terms.push_back(qt::AccTerm{ptr_of(c, s.H), ptr_of(c, s.X)});
  std::vector<qt::LinTask> lin;
  for (auto& s : P.lin) {
    qt::LinTask t;
    t.out = mptr_of(c, s.out);
    t.d = s.d;
    t.first = s.first;
    t.count = s.count;
    t.pad = 0;
    lin.push_back(t);
  }
  std::vector<qt::LinTerm> lin_terms;
  for (auto& s : P.lin_terms) lin_terms.push_back(qt::LinTerm{s.c, ptr_of(c, s.M)});
  std::vector<qt::EigTask> eig;
  for (auto& s : P.eig) {
    qt::EigTask t;
    t.rho = ptr_of(c, s.rho);
    t.rhoinv = mptr_of(c, s.rhoinv);
    t.U = mptr_of(c, s.U);
    t.d = s.d;
    t.pad = 0;
    eig.push_back(t);
  }
  std::vector<qt::ProjTask> proj;
  for (auto& s : P.proj) {
    qt::ProjTask t;
    t.S = mptr_of(c, s.S);
    t.D = ptr_of(c, s.D);
    t.rhoinv = ptr_of(c, s.rhoinv);
    t.Sinv = mptr_of(c, s.Sinv);
    t.P = mptr_of(c, s.P);
    t.M2 = mptr_of(c, s.M2);
    t.d = s.d;
    t.pad = 0;
    proj.push_back(t);
  }
  std::vector<qt::CvtTask> cvt;
  for (auto& s : P.cvt) {
    qt::CvtTask t;
    t.src = ptr_of(c, s.src);
    t.dst = mptr_of(c, s.dst);
    t.n = s.n;
    t.dir = s.dir;
    t.pad = 0;
    cvt.push_back(t);
  }
  std::vector<qt::GradTask> gtasks;
  for (auto& s : P.grad) {
    qt::GradTask t;
    t.eout = ptr_of(c, s.eout);
    t.rho = ptr_of(c, s.rho);
    t.m3 = mptr_of(c, s.m3);
    t.h00 = ptr_of(c, s.h00);
    t.s00 = ptr_of(c, s.s00);
    t.alpha = mptr_of(c, s.alpha);
    t.d = s.d;
    t.write_alpha = s.write_alpha;
    gtasks.push_back(t);
  }
  std::vector<qt::MMTask> mmt;
  for (auto& m : P.mm) mmt.push_back(qt::MMTask{mptr_of(c, m.out), m.d, m.first, m.count, m.trans_b});
  std::vector<qt::MMTerm> mmterms;
  for (auto& m : P.mm_terms) mmterms.push_back(qt::MMTerm{ptr_of(c, m.A), ptr_of(c, m.B)});
  // CDVR tables
  std::vector<qt::TCTask> tct;
  for (auto& x : P.tc) {
    qt::TCTask t;
    t.A = ptr_of(c, x.A);
    t.B = ptr_of(c, x.B);
    t.C = mptr_of(c, x.C);
    t.alpha = x.alpha;
    t.M0 = x.M0;
    t.M1 = x.M1;
    t.N0 = x.N0;
    t.N1 = x.N1;
    t.K0 = x.K0;
    t.K1 = x.K1;
    t.conjA = x.conjA;
    t.conjB = x.conjB;
    t.add = x.add;
    t.pad = 0;
    t.am0 = x.am0;
    t.am1 = x.am1;
    t.ak0 = x.ak0;
    t.ak1 = x.ak1;
    t.bk0 = x.bk0;
    t.bk1 = x.bk1;
    t.bn0 = x.bn0;
    t.bn1 = x.bn1;
    t.cm0 = x.cm0;
    t.cm1 = x.cm1;
    t.cn0 = x.cn0;
    t.cn1 = x.cn1;
    tct.push_back(t);
  }
  std::vector<qt::GSTask> gst;
  for (auto& x : P.gs) gst.push_back(qt::GSTask{ptr_of(c, x.in), ptr_of(c, x.noise), mptr_of(c, x.out), x.rows, x.cols});
  std::vector<qt::EigFTask> eft;
  for (auto& x : P.eigf)
    eft.push_back(qt::EigFTask{ptr_of(c, x.A), mptr_of(c, x.out), mptr_of(c, x.U), mptr_of(c, x.W), mptr_of(c, x.vals),
                               x.eps, x.d, x.fn});
  std::vector<qt::WSDTask> wst;
  for (auto& x : P.wsd)
    wst.push_back(qt::WSDTask{ptr_of(c, x.W), mptr_of(c, x.trafo), mptr_of(c, x.grid), mptr_of(c, x.scratch), x.d, x.n,
                              x.first, 0});
  std::vector<qt::WSDTerm> wsterms;
  for (auto& x : P.wsd_terms) wsterms.push_back(qt::WSDTerm{ptr_of(c, x)});
  std::vector<qt::VPotTask> vpt;
  for (auto& x : P.vpot) {
    qt::VPotTask t;
    t.out = mptr_of(c, x.out);
    t.n = x.n;
    t.order = x.order;
    t.first = x.first;
    for (int i = 0; i < 6; ++i) t.dims[i] = x.dims[i];
    vpt.push_back(t);
  }
  std::vector<qt::VCoord> vco;
  for (auto& x : P.vcoords) vco.push_back(qt::VCoord{ptr_of(c, x.grid), x.index, 0});
  std::vector<qt::PotTerm> pterms;
  std::vector<qt::PotFactor> pfacts;
  if (P.cdvr) {
    for (size_t q = 0; q < c->cdvr.coeff.size(); ++q)
      pterms.push_back(qt::PotTerm{c->cdvr.coeff[q], c->cdvr.ptr[q], c->cdvr.ptr[q + 1] - c->cdvr.ptr[q]});
    for (size_t q = 0; q < c->cdvr.mode.size(); ++q) pfacts.push_back(qt::PotFactor{c->cdvr.mode[q], c->cdvr.power[q]});
  }
  std::vector<qt::DVLTask> dvt;
  for (auto& x : P.dvl)
    dvt.push_back(qt::DVLTask{ptr_of(c, x.cup), ptr_of(c, x.vnode), ptr_of(c, x.vedge), mptr_of(c, x.dv), x.bef, x.d});
  std::vector<qt::EWTask> ewt;
  for (auto& x : P.ew) ewt.push_back(qt::EWTask{ptr_of(c, x.v), ptr_of(c, x.in), mptr_of(c, x.out), x.n, x.add, 0});
  std::vector<char> blob;
  std::vector<int64_t> offs;
  put(blob, offs, mp);
  put(blob, offs, hp);
  put(blob, offs, acc);
  put(blob, offs, acc_terms);
  put(blob, offs, lin);
  put(blob, offs, lin_terms);
  put(blob, offs, eig);
  put(blob, offs, proj);
  put(blob, offs, P.mp_tiles);
  put(blob, offs, P.hp_tiles);
  put(blob, offs, P.acc_tiles);
  put(blob, offs, cvt);
  put(blob, offs, P.cvt_tiles);
  put(blob, offs, gtasks);
  put(blob, offs, mmt);
  put(blob, offs, mmterms);
  put(blob, offs, P.mm_tiles);
  put(blob, offs, tct);
  put(blob, offs, P.tc_tiles);
  put(blob, offs, gst);
  put(blob, offs, eft);
  put(blob, offs, wst);
  put(blob, offs, wsterms);
  put(blob, offs, vpt);
  put(blob, offs, vco);
  put(blob, offs, P.vpot_tiles);
  put(blob, offs, pterms);
  put(blob, offs, pfacts);
  put(blob, offs, dvt);
  put(blob, offs, P.dvl_tiles);
  put(blob, offs, ewt);
  put(blob, offs, P.ew_tiles);
  put(blob, offs, P.mp_oz_tiles);
  put(blob, offs, P.mp_oz_tasks);
  put(blob, offs, hp_tc);
  put(blob, offs, P.hp_tc_items);
  put(blob, offs, P.hp_tc_imgs);
  put(blob, offs, P.acc_tc_items);
  put(blob, offs, P.acc_tc_imgs);
  {
    cudaError_t e = dev_malloc(&c->tables_mem, std::max<size_t>(blob.size(), 256));
    if (e != cudaSuccess) {
      release_arena(c);
      return fail(c, QT_ERR_ALLOC, std::string("qt_prepare: task table allocation failed: ") + cudaGetErrorString(e));
    }
    arena += (int64_t)blob.size();
  }
  QT_CUDA(c, cudaMemcpyAsync(c->tables_mem, blob.data(), blob.size(), cudaMemcpyHostToDevice, c->stream));
  char* base = (char*)c->tables_mem;
  c->tables.mp = (qt::MPTask*)(base + offs[0]);
  c->tables.hp = (qt::HPTask*)(base + offs[1]);
  c->tables.acc = (qt::AccTask*)(base + offs[2]);
  c->tables.acc_terms = (qt::AccTerm*)(base + offs[3]);
  c->tables.lin = (qt::LinTask*)(base + offs[4]);
  c->tables.lin_terms = (qt::LinTerm*)(base + offs[5]);
  c->tables.eig = (qt::EigTask*)(base + offs[6]);
  c->tables.proj = (qt::ProjTask*)(base + offs[7]);
  c->tables.mp_tiles = (int2*)(base + offs[8]);
  c->tables.hp_tiles = (int4*)(base + offs[9]);
  c->tables.hp_ws = c->buf[qt::B_HPW];
  c->tables.hp_segs = P.hp_segs.data();
  c->tables.acc_tiles = (int4*)(base + offs[10]);
  c->tables.cvt = (qt::CvtTask*)(base + offs[11]);
  c->tables.cvt_tiles = (int2*)(base + offs[12]);
  c->tables.grad = (qt::GradTask*)(base + offs[13]);
  c->tables.mm = (qt::MMTask*)(base + offs[14]);
  c->tables.mm_terms = (qt::MMTerm*)(base + offs[15]);
  c->tables.mm_tiles = (int2*)(base + offs[16]);
  c->tables.tc = (qt::TCTask*)(base + offs[17]);
  c->tables.tc_tiles = (int4*)(base + offs[18]);
  c->tables.gs = (qt::GSTask*)(base + offs[19]);
  c->tables.eigf = (qt::EigFTask*)(base + offs[20]);
  c->tables.wsd = (qt::WSDTask*)(base + offs[21]);
  c->tables.wsd_terms = (qt::WSDTerm*)(base + offs[22]);
  c->tables.vpot = (qt::VPotTask*)(base + offs[23]);
  c->tables.vcoords = (qt::VCoord*)(base + offs[24]);
  c->tables.vpot_tiles = (int2*)(base + offs[25]);
  c->tables.pot_terms = (qt::PotTerm*)(base + offs[26]);
  c->tables.pot_factors = (qt::PotFactor*)(base + offs[27]);
  c->tables.n_pot_terms = (int)pterms.size();
  c->tables.n_modes = (int)c->cdvr.leaf_x.size();
  c->tables.wsd_max_n = P.wsd_max_n;
  c->tables.wsd_max_d = P.wsd_max_d;
  c->tables.dvl = (qt::DVLTask*)(base + offs[28]);
  c->tables.dvl_tiles = (int2*)(base + offs[29]);
  c->tables.ew = (qt::EWTask*)(base + offs[30]);
  c->tables.ew_tiles = (int2*)(base + offs[31]);
  c->tables.status = reinterpret_cast<int*>(c->buf[qt::B_PARAM] + 15);
  c->tables.mp_oz_tiles = (int2*)(base + offs[32]);
  c->tables.mp_oz_tasks = (int*)(base + offs[33]);
  c->tables.hp_tc_groups = (qt::HpTcGroup*)(base + offs[34]);
  c->tables.hp_tc_items = (int4*)(base + offs[35]);
  c->tables.hp_tc_imgs = (int2*)(base + offs[36]);
  c->tables.acc_tc_items = (int4*)(base + offs[37]);
  c->tables.acc_tc_imgs = (int2*)(base + offs[38]);
  if (P.cdvr) {  // CDVR constants: seeded noise, leaf grids, identity
    QT_CUDA(c, cudaMemsetAsync(c->buf[qt::B_CDVR], 0, c->buf_elems[qt::B_CDVR] * 16, c->stream));
    for (auto& init : P.cdvr_init)
      QT_CUDA(c, cudaMemcpyAsync(c->buf[qt::B_CDVR] + init.first, init.second.data(), init.second.size() * 16,
                                 cudaMemcpyHostToDevice, c->stream));
  }
  for (auto& id : P.identities) {
    cudaError_t e = qt::launch_set_identity(c->buf[qt::B_MATS] + id.first, id.second, prec, c->stream);
    if (e != cudaSuccess) return cuda_fail(c, e, "set identity");
    c->launches += 1;
  }
  QT_CUDA(c, cudaStreamSynchronize(c->stream));
  // capture the sweep
  QT_CUDA(c, cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
  for (int64_t i = 0; i < P.main_end; ++i) {
    const auto& st = P.stages[i];
    cudaError_t e = qt::launch_stage(st, c->tables, c->eps, P.max_eig_d, prec, c->stream);
    if (e != cudaSuccess) {
      cudaGraph_t g = nullptr;
      cudaStreamEndCapture(c->stream, &g);
      if (g) cudaGraphDestroy(g);
      release_arena(c);
      return cuda_fail(c, e, (std::string("capture stage ") + st.name).c_str());
    }
  }
  QT_CUDA(c, cudaStreamEndCapture(c->stream, &c->graph));
  QT_CUDA(c, cudaGraphInstantiate(&c->exec, c->graph, 0));
  // the same stages split into build / frozen-matrix derivative graphs (CMF)
  for (int part = 0; part < 2; ++part) {
    QT_CUDA(c, cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
    cudaError_t e = cudaSuccess;
    const bool own = P.main_end < (int64_t)P.stages.size();  // separate frozen-matrix stages
    const int64_t b0 = part == 0 ? 0 : (own ? P.main_end : P.apply_begin);
    const int64_t b1 = part == 0 ? P.apply_begin : (own ? (int64_t)P.stages.size() : P.main_end);
    if (part == 1 && prec >= 1) e = qt::launch_stage(P.stages[0], c->tables, c->eps, P.max_eig_d, prec, c->stream);
    for (int64_t i = b0; i < b1 && e == cudaSuccess; ++i)
      e = qt::launch_stage(P.stages[i], c->tables, c->eps, P.max_eig_d, prec, c->stream);
    cudaGraph_t g = nullptr;
    cudaError_t e2 = cudaStreamEndCapture(c->stream, &g);
    if (e == cudaSuccess) e = e2;
    if (e == cudaSuccess) e = cudaGraphInstantiate(part == 0 ? &c->exec_build : &c->exec_apply, g, 0);
    if (g) cudaGraphDestroy(g);
    if (e != cudaSuccess) {
      release_arena(c);
      return cuda_fail(c, e, "capture of the build / apply graphs");
    }
  }
  P.stats.arena_bytes = arena;
  P.stats.scratch_bytes = c->buf_elems[qt::B_SCR] * 16;
  c->prepared = true;
  return QT_OK;
}

int64_t qt_psi_size(const qt_ctx* c) { return (c && c->prepared) ? c->plan.psi_packed : -1; }

int qt_psi_upload(qt_ctx* c, const double* psi) {
  if (!c || !psi) return fail(c, QT_ERR_ARG, "null argument");
  QT_DEVICE(c);
  if (!c->prepared) return fail(c, QT_ERR_STATE, "qt_psi_upload before qt_prepare");
  QT_CUDA(c, cudaMemcpyAsync(c->buf[qt::B_PSI64], psi, c->plan.psi_packed * 16, cudaMemcpyHostToDevice,
                             c->stream));
  c->have_psi = true;
  c->swept = false;
  return QT_OK;
}

int qt_psi_upload_device(qt_ctx* c, const void* psi) {
  if (!c || !psi) return fail(c, QT_ERR_ARG, "null argument");
  QT_DEVICE(c);
  if (!c->prepared) return fail(c, QT_ERR_STATE, "qt_psi_upload_device before qt_prepare");
  QT_CUDA(c, cudaMemcpyAsync(c->buf[qt::B_PSI64], psi, c->plan.psi_packed * 16, cudaMemcpyDeviceToDevice,
                             c->stream));
  c->have_psi = true;
  c->swept = false;
  return QT_OK;
}

int qt_psi_download(qt_ctx* c, double* psi) {
  if (!c || !psi) return fail(c, QT_ERR_ARG, "null argument");
  QT_DEVICE(c);
  if (!c->have_psi) return fail(c, QT_ERR_STATE, "no wavefunction uploaded");
  QT_CUDA(c, cudaMemcpyAsync(psi, c->buf[qt::B_PSI64], c->plan.psi_packed * 16, cudaMemcpyDeviceToHost,
                             c->stream));
  QT_CUDA(c, cudaStreamSynchronize(c->stream));
  return QT_OK;
}

int qt_psi_save(qt_ctx* c, const char* path) {
  if (!c || !path) return fail(c, QT_ERR_ARG, "null argument");
  QT_DEVICE(c);
  if (!c->have_psi) return fail(c, QT_ERR_STATE, "no wavefunction uploaded");
  std::vector<double2> psi(c->plan.psi_packed);
  QT_CUDA(c, cudaMemcpyAsync(psi.data(), c->buf[qt::B_PSI64], psi.size() * 16, cudaMemcpyDeviceToHost,
                             c->stream));
  QT_CUDA(c, cudaStreamSynchronize(c->stream));
  FILE* f = std::fopen(path, "wb");
  if (!f) return fail(c, QT_ERR_ARG, std::string("qt_psi_save: cannot open ") + path);
  const int32_t nn = (int32_t)c->plan.nodes.size();
  bool ok = std::fwrite("TTre", 1, 4, f) == 4 && std::fwrite(&nn, 4, 1, f) == 1;
  for (const auto& g : c->plan.nodes) {
    const int32_t order = (int32_t)g.shape.size(), sz = 16;
    ok = ok && std::fwrite("TENS", 1, 4, f) == 4 && std::fwrite("TDIM", 1, 4, f) == 4 &&
         std::fwrite(&order, 4, 1, f) == 1;
    for (int d : g.shape) {
      const int32_t v = d;
      ok = ok && std::fwrite(&v, 4, 1, f) == 1;
    }
    ok = ok && std::fwrite(&sz, 4, 1, f) == 1 &&
         std::fwrite(psi.data() + g.off, 16, (size_t)g.N, f) == (size_t)g.N;
  }
  ok = (std::fclose(f) == 0) && ok;
  if (!ok) return fail(c, QT_ERR_ARG, std::string("qt_psi_save: write failed for ") + path);
  return QT_OK;
}

int qt_psi_load(qt_ctx* c, const char* path) {
  if (!c || !path) return fail(c, QT_ERR_ARG, "null argument");
  QT_DEVICE(c);
  if (!c->prepared) return fail(c, QT_ERR_STATE, "qt_psi_load before qt_prepare");
  FILE* f = std::fopen(path, "rb");
  if (!f) return fail(c, QT_ERR_ARG, std::string("qt_psi_load: cannot open ") + path);
  std::vector<double2> psi(c->plan.psi_packed);
  char tag[4];
  int32_t nn = 0;
  std::string err;
  if (std::fread(tag, 1, 4, f) != 4 || std::memcmp(tag, "TTre", 4) != 0) err = "not a TTre file";
  if (err.empty() && (std::fread(&nn, 4, 1, f) != 1 || nn != (int32_t)c->plan.nodes.size()))
    err = "node count differs from the tree";
  for (size_t i = 0; err.empty() && i < c->plan.nodes.size(); ++i) {
    const auto& g = c->plan.nodes[i];
    int32_t order = 0, sz = 0;
    if (std::fread(tag, 1, 4, f) != 4 || std::memcmp(tag, "TENS", 4) != 0) { err = "missing TENS"; break; }
    if (std::fread(tag, 1, 4, f) != 4 || std::memcmp(tag, "TDIM", 4) != 0) { err = "missing TDIM"; break; }
    if (std::fread(&order, 4, 1, f) != 1 || order != (int32_t)g.shape.size()) { err = "node order differs"; break; }
    for (int k = 0; k < order; ++k) {
      int32_t d = 0;
      if (std::fread(&d, 4, 1, f) != 1 || d != g.shape[k]) { err = "node shape differs"; break; }
    }
    if (!err.empty()) break;
    if (std::fread(&sz, 4, 1, f) != 1 || sz != 16) { err = "element size is not complex128"; break; }
    if (std::fread(psi.data() + g.off, 16, (size_t)g.N, f) != (size_t)g.N) { err = "file truncated"; break; }
  }
  std::fclose(f);
  if (!err.empty()) return fail(c, QT_ERR_SHAPE, std::string("qt_psi_load: ") + err + " (" + path + ")");
  if (!finite_all((const double*)psi.data(), 2 * (int64_t)psi.size()))
    return fail(c, QT_ERR_NUMERIC, "qt_psi_load: non-finite coefficient");
  QT_CUDA(c, cudaMemcpyAsync(c->buf[qt::B_PSI64], psi.data(), psi.size() * 16, cudaMemcpyHostToDevice,
                             c->stream));
  QT_CUDA(c, cudaStreamSynchronize(c->stream));
  c->have_psi = true;
  c->swept = false;
  return QT_OK;
}

namespace {
// kernel launches of stages [b0, b1): a hole-product stage one per tile
// shape, two for its tensor-core items (image pre-pass and products), one
// for the partial sums of split tasks; a mode-product stage one for its
// FP32-pipe tiles and two for its tensor-core tiles (pre-pass and products)
int64_t kernels_in(const qt::Plan& P, int64_t b0, int64_t b1) {
  int64_t n = 0;
  for (int64_t i = b0; i < b1; ++i) {
    const qt::Stage& st = P.stages[i];
    if (st.kind == qt::ST_HP)
      n += st.nseg + (st.nhti > 0 ? (st.nhtu > 0 ? 3 : 2) : 0) + (st.aux ? 1 : 0);
    else if (st.kind == qt::ST_MP)
      n += (st.n_tiles > 0 ? 1 : 0) + (st.noz > 0 ? (st.nozt > 0 ? 2 : 1) : 0);
    else if (st.kind == qt::ST_ACC)
      n += (st.n_tiles > 0 ? 1 : 0) + (st.nati > 0 ? (st.natu > 0 ? 2 : 1) : 0);
    else
      n += 1;
  }
  return n;
}
// launches of one frozen-matrix derivative graph
int64_t apply_launches(const qt_ctx* c) {
  const qt::Plan& P = c->plan;
  const int64_t n = P.main_end < (int64_t)P.stages.size() ? kernels_in(P, P.main_end, (int64_t)P.stages.size())
                                                          : kernels_in(P, P.apply_begin, P.main_end);
  return n + (c->prec >= 1 ? 1 : 0);
}
}  // namespace

int qt_derivative(qt_ctx* c, double phase_re, double phase_im) {
  if (!c) return fail(c, QT_ERR_ARG, "null context");
  QT_DEVICE(c);
  if (!c->prepared || !c->have_psi) return fail(c, QT_ERR_STATE, "qt_derivative needs qt_prepare and a wavefunction");
  // alpha = -i * phase
  double2 alpha = make_double2(phase_im, -phase_re);
  QT_CUDA(c, cudaMemcpyAsync(c->buf[qt::B_PARAM], &alpha, sizeof(double2), cudaMemcpyHostToDevice, c->stream));
  QT_CUDA(c, cudaGraphLaunch(c->exec, c->stream));
  c->launches += kernels_in(c->plan, 0, c->plan.main_end);
  c->swept = true;
  c->built = true;
  return QT_OK;
}

int qt_build(qt_ctx* c) {
  if (!c) return fail(c, QT_ERR_ARG, "null context");
  QT_DEVICE(c);
  if (!c->prepared || !c->have_psi) return fail(c, QT_ERR_STATE, "qt_build needs qt_prepare and a wavefunction");
  QT_CUDA(c, cudaGraphLaunch(c->exec_build, c->stream));
  c->launches += kernels_in(c->plan, 0, c->plan.apply_begin);
  c->built = true;
  return QT_OK;
}

int qt_layer_derivatives(qt_ctx* c, double phase_re, double phase_im) {
  if (!c) return fail(c, QT_ERR_ARG, "null context");
  QT_DEVICE(c);
  if (!c->prepared || !c->have_psi || !c->built)
    return fail(c, QT_ERR_STATE, "qt_layer_derivatives needs a qt_build (or qt_derivative) first");
  double2 alpha = make_double2(phase_im, -phase_re);
  QT_CUDA(c, cudaMemcpyAsync(c->buf[qt::B_PARAM], &alpha, sizeof(double2), cudaMemcpyHostToDevice, c->stream));
  QT_CUDA(c, cudaGraphLaunch(c->exec_apply, c->stream));
  c->launches += apply_launches(c);
  c->swept = true;
  return QT_OK;
}

namespace {
// RK4 with the matrices of the last build frozen, from Y over `steps` steps of
// length h; uses B_PSI64 as the derivative input and ACC as workspace.
int rk4_frozen(qt_ctx* c, double2* Y, double2* ACC, double h, int steps, double2 alpha) {
  const int64_t n = c->plan.psi_packed;
  double2* IN = c->buf[qt::B_PSI64];
  const double2* K = c->buf[qt::B_DPSI64];
  const double2 one = make_double2(1.0, 0.0);
  for (int s = 0; s < steps; ++s) {
    const double w[4] = {1.0, 2.0, 2.0, 1.0};
    const double a[4] = {0.5 * h, 0.5 * h, h, 0.0};
    QT_CUDA(c, cudaMemcpyAsync(IN, Y, n * 16, cudaMemcpyDeviceToDevice, c->stream));
    for (int k = 0; k < 4; ++k) {
      QT_CUDA(c, cudaMemcpyAsync(c->buf[qt::B_PARAM], &alpha, sizeof(double2), cudaMemcpyHostToDevice, c->stream));
      QT_CUDA(c, cudaGraphLaunch(c->exec_apply, c->stream));
      c->launches += apply_launches(c);
      cudaError_t e = k == 0 ? cudaMemcpyAsync(ACC, K, n * 16, cudaMemcpyDeviceToDevice, c->stream)
                             : qt::launch_axpy(ACC, ACC, make_double2(w[k], 0.0), K, n, c->stream);
      if (e != cudaSuccess) return cuda_fail(c, e, "rk4 accumulate");
      if (k < 3) {
        e = qt::launch_axpy(IN, Y, make_double2(a[k], 0.0), K, n, c->stream);
        if (e != cudaSuccess) return cuda_fail(c, e, "rk4 stage");
      }
      c->launches += 2;
    }
    cudaError_t e = qt::launch_axpy(Y, Y, make_double2(h / 6.0, 0.0), ACC, n, c->stream);
    if (e != cudaSuccess) return cuda_fail(c, e, "rk4 update");
    c->launches += 1;
    (void)one;
  }
  return QT_OK;
}
}  // namespace

int qt_cmf_propagate(qt_ctx* c, double dt, int n_steps, int n_sub, double phase_re, double phase_im) {
  if (!c) return fail(c, QT_ERR_ARG, "null context");
  if (!c->prepared || !c->have_psi) return fail(c, QT_ERR_STATE, "qt_cmf_propagate needs qt_prepare and a wavefunction");
  if (!(dt > 0) || !std::isfinite(dt) || n_steps < 0 || n_sub < 1)
    return fail(c, QT_ERR_ARG, "qt_cmf_propagate: need dt > 0, n_steps >= 0, n_sub >= 1");
  QT_DEVICE(c);
  const int64_t n = c->plan.psi_packed;
  for (auto& b : c->cmf_buf)
    if (!b) {
      cudaError_t e = dev_malloc((void**)&b, n * 16);
      if (e != cudaSuccess) return fail(c, QT_ERR_ALLOC, "qt_cmf_propagate: work vectors");
    }
  double2* Y0 = c->cmf_buf[0];
  double2* Y = c->cmf_buf[1];
  double2* ACC = c->cmf_buf[2];
  double2* PSI = c->buf[qt::B_PSI64];
  const double2 alpha = make_double2(phase_im, -phase_re);  // -i * phase
  for (int step = 0; step < n_steps; ++step) {
    QT_CUDA(c, cudaMemcpyAsync(Y0, PSI, n * 16, cudaMemcpyDeviceToDevice, c->stream));
    // matrices at t, propagate to t + dt/2
    QT_CUDA(c, cudaGraphLaunch(c->exec_build, c->stream));
    QT_CUDA(c, cudaMemcpyAsync(Y, Y0, n * 16, cudaMemcpyDeviceToDevice, c->stream));
    int rc = rk4_frozen(c, Y, ACC, 0.5 * dt / n_sub, n_sub, alpha);
    if (rc != QT_OK) return rc;
    // matrices at t + dt/2, propagate Psi(t) over the full step
    QT_CUDA(c, cudaMemcpyAsync(PSI, Y, n * 16, cudaMemcpyDeviceToDevice, c->stream));
    QT_CUDA(c, cudaGraphLaunch(c->exec_build, c->stream));
    QT_CUDA(c, cudaMemcpyAsync(Y, Y0, n * 16, cudaMemcpyDeviceToDevice, c->stream));
    rc = rk4_frozen(c, Y, ACC, 0.5 * dt / n_sub, 2 * n_sub, alpha);
    if (rc != QT_OK) return rc;
    QT_CUDA(c, cudaMemcpyAsync(PSI, Y, n * 16, cudaMemcpyDeviceToDevice, c->stream));
    c->launches += 2 * kernels_in(c->plan, 0, c->plan.apply_begin);
  }
  c->built = false;
  c->swept = false;
  return QT_OK;
}

int qt_dpsi_download(qt_ctx* c, double* out) {
  if (!c || !out) return fail(c, QT_ERR_ARG, "null argument");
  QT_DEVICE(c);
  if (!c->swept) return fail(c, QT_ERR_STATE, "no sweep has run");
  QT_CUDA(c, cudaMemcpyAsync(out, c->buf[qt::B_DPSI64], c->plan.psi_packed * 16, cudaMemcpyDeviceToHost,
                             c->stream));
  QT_CUDA(c, cudaStreamSynchronize(c->stream));
  return check_status(c);
}

int qt_gradient_download(qt_ctx* c, double* out) {
  if (!c || !out) return fail(c, QT_ERR_ARG, "null argument");
  QT_DEVICE(c);
  if (!c->swept) return fail(c, QT_ERR_STATE, "no sweep has run");
  if (!c->plan.want_grad) return fail(c, QT_ERR_STATE, "plan prepared without QT_PLAN_GRADIENT");
  QT_CUDA(c, cudaMemcpyAsync(out, c->buf[qt::B_GRAD64], c->plan.psi_packed * 16, cudaMemcpyDeviceToHost,
                             c->stream));
  QT_CUDA(c, cudaStreamSynchronize(c->stream));
  return QT_OK;
}

int qt_dpsi_device(qt_ctx* c, const void** p) {
  if (!c || !p) return fail(c, QT_ERR_ARG, "null argument");
  if (!c->prepared) return fail(c, QT_ERR_STATE, "qt_dpsi_device before qt_prepare");
  *p = c->buf[qt::B_DPSI64];
  return QT_OK;
}

int qt_energy(qt_ctx* c, double* out4) { return qt_energies(c, out4, 1); }

int qt_tree_count(const qt_ctx* c) { return (c && c->prepared) ? (int)c->plan.tops.size() : -1; }

int qt_energies(qt_ctx* c, double* out, int n_trees) {
  if (!c || !out) return fail(c, QT_ERR_ARG, "null argument");
  QT_DEVICE(c);
  if (!c->swept) return fail(c, QT_ERR_STATE, "no sweep has run");
  const int nt = (int)c->plan.tops.size();
  if (n_trees < 1 || n_trees > nt) return fail(c, QT_ERR_ARG, "qt_energies: n_trees out of range");
  std::vector<double2> v(2 * (size_t)n_trees);
  for (int k = 0; k < n_trees; ++k) {
    QT_CUDA(c, cudaMemcpyAsync(&v[2 * k], c->buf[qt::B_MATS] + c->plan.energy_off[k], 16,
                               cudaMemcpyDeviceToHost, c->stream));
    QT_CUDA(c, cudaMemcpyAsync(&v[2 * k + 1], c->buf[qt::B_MATS] + c->plan.stop_off[k], 16,
                               cudaMemcpyDeviceToHost, c->stream));
  }
  QT_CUDA(c, cudaStreamSynchronize(c->stream));
  if (int st = check_status(c)) return st;
  for (int k = 0; k < n_trees; ++k) {
    out[4 * k + 0] = v[2 * k].x;
    out[4 * k + 1] = v[2 * k].y;
    out[4 * k + 2] = v[2 * k + 1].x;
    out[4 * k + 3] = v[2 * k + 1].y;
  }
  if (!finite_all(out, 4 * (int64_t)n_trees)) return fail(c, QT_ERR_NUMERIC, "non-finite energy");
  return QT_OK;
}

int64_t qt_matrices_size(const qt_ctx* c, int which) {
  if (!c || !c->prepared) return -1;
  const Plan& P = c->plan;
  int64_t s = 0;
  int n = (int)P.nodes.size();
  if (which == QT_MAT_RHO || which == QT_MAT_RHOINV) {
    for (int a = 0; a < n; ++a) s += (int64_t)P.nodes[a].dup() * P.nodes[a].dup();
    return s;
  }
  if (which == QT_MAT_HMAT || which == QT_MAT_HCON) {
    for (const auto& nodes : P.term_nodes)
      for (int a : nodes) s += (int64_t)P.nodes[a].dup() * P.nodes[a].dup();
    return s;
  }
  if (which == QT_MAT_CDVR) return P.cdvr ? P.cdvr_size : -1;
  return -1;
}

int qt_matrices_download(qt_ctx* c, int which, double* out) {
  if (!c || !out) return fail(c, QT_ERR_ARG, "null argument");
  QT_DEVICE(c);
  // the build graph writes every matrix set; a sweep runs it too
  if (!c->swept && !c->built) return fail(c, QT_ERR_STATE, "no sweep or qt_build has run");
  const Plan& P = c->plan;
  if (which == QT_MAT_CDVR) {
    if (!P.cdvr) return fail(c, QT_ERR_STATE, "plan prepared without QT_PLAN_CDVR");
    QT_CUDA(c, cudaMemcpyAsync(out, c->buf[qt::B_CDVR], P.cdvr_size * 16, cudaMemcpyDeviceToHost, c->stream));
    QT_CUDA(c, cudaStreamSynchronize(c->stream));
    return QT_OK;
  }
  if ((which == QT_MAT_HMAT || which == QT_MAT_HCON) && !P.per_term_mats)
    return fail(c, QT_ERR_STATE, "the compressed plan keeps no per-term matrices");
  std::vector<double2> mats(P.mats_size);
  QT_CUDA(c, cudaMemcpyAsync(mats.data(), c->buf[qt::B_MATS], P.mats_size * 16, cudaMemcpyDeviceToHost, c->stream));
  QT_CUDA(c, cudaStreamSynchronize(c->stream));
  double2* o = (double2*)out;
  int n = (int)P.nodes.size();
  int64_t cur = 0;
  if (c->prec >= 1 && (which == QT_MAT_HMAT || which == QT_MAT_HCON)) {
    // double-float slots -> complex128
    for (auto& v : mats) {
      float4 f;
      std::memcpy(&f, &v, 16);
      v = make_double2((double)f.x + (double)f.y, (double)f.z + (double)f.w);
    }
  }
  if (which == QT_MAT_RHO || which == QT_MAT_RHOINV) {
    const auto& off = which == QT_MAT_RHO ? P.rho64_off : P.rhoinv64_off;
    for (int a = 0; a < n; ++a) {
      int64_t dd = (int64_t)P.nodes[a].dup() * P.nodes[a].dup();
      std::memcpy(o + cur, mats.data() + off[a], dd * 16);
      cur += dd;
    }
    return QT_OK;
  }
  if (which == QT_MAT_HMAT || which == QT_MAT_HCON) {
    const auto& slot = which == QT_MAT_HMAT ? P.term_hslot : P.term_cslot;
    for (size_t l = 0; l < P.term_nodes.size(); ++l)
      for (size_t i = 0; i < P.term_nodes[l].size(); ++i) {
        const int a = P.term_nodes[l][i];
        int64_t dd = (int64_t)P.nodes[a].dup() * P.nodes[a].dup();
        if (slot[l][i] >= 0)
          std::memcpy(o + cur, mats.data() + slot[l][i], dd * 16);
        else
          std::memset((void*)(o + cur), 0, dd * 16);
        cur += dd;
      }
    return QT_OK;
  }
  return fail(c, QT_ERR_ARG, "unknown matrix set");
}

int qt_plan_stats(const qt_ctx* c, double* out) {
  if (!c || !out) return QT_ERR_ARG;
  if (!c->prepared) return QT_ERR_STATE;
  const auto& s = c->plan.stats;
  out[0] = s.ref_flops;
  out[1] = s.exec_flops;
  out[2] = (double)c->plan.main_end;
  out[3] = (double)s.arena_bytes;
  out[4] = (double)s.scratch_bytes;
  out[5] = (double)s.rep_chains;
  out[6] = (double)s.mf_chains;
  out[7] = (double)s.app_chains;
  return QT_OK;
}

int qt_mode_product(qt_ctx* c, void* C, const void* h, const void* B, int64_t before, int64_t activeB,
                    int64_t activeC, int64_t after, int add) {
  if (!c || !C || !h || !B) return fail(c, QT_ERR_ARG, "qt_mode_product: null argument");
  if (before < 1 || activeB < 1 || activeC < 1 || after < 1 || before * activeB * after > ((int64_t)1 << 31) ||
      before * activeC * after > ((int64_t)1 << 31))
    return fail(c, QT_ERR_SHAPE, "qt_mode_product: bad geometry");
  if (C == B) return fail(c, QT_ERR_ARG, "qt_mode_product: C must not alias B");
  QT_DEVICE(c);
  qt::MPTask t;
  t.in = (const double2*)B;
  t.out = (double2*)C;
  t.h = (const double2*)h;
  t.alpha = make_double2(1.0, 0.0);
  t.before = (int)before;
  t.a_in = (int)activeB;
  t.a_out = (int)activeC;
  t.after = (int)after;
  t.diag = 0;
  t.add = add ? 1 : 0;
  cudaError_t e = qt::launch_single_mp(t, c->stream, nullptr);
  if (e != cudaSuccess) return cuda_fail(c, e, "qt_mode_product");
  c->launches += 1;
  return QT_OK;
}

int qt_hole_product(qt_ctx* c, void* S, const void* A, const void* B, int64_t before, int64_t activeA,
                    int64_t activeB, int64_t after) {
  if (!c || !S || !A || !B) return fail(c, QT_ERR_ARG, "qt_hole_product: null argument");
  if (before < 1 || activeA < 1 || activeB < 1 || after < 1 || before * activeA * after > ((int64_t)1 << 31) ||
      before * activeB * after > ((int64_t)1 << 31) || activeA + activeB > 800)
    return fail(c, QT_ERR_SHAPE, "qt_hole_product: bad geometry");
  QT_DEVICE(c);
  qt::HPTask t;
  t.A = (const double2*)A;
  t.B = (const double2*)B;
  t.S = (double2*)S;
  t.before = (int)before;
  t.a = (int)activeA;
  t.after = (int)after;
  t.aB = (int)activeB;
  t.splits = 1;
  t.kchunk = 0;
  t.ws = 0;
  t.rows = t.cols = 4;
  cudaError_t e = qt::launch_single_hp(t, c->stream, nullptr);
  if (e != cudaSuccess) return cuda_fail(c, e, "qt_hole_product");
  c->launches += 1;
  return QT_OK;
}

int qt_last_mode_product(qt_ctx* c, void* C, const void* A, const void* B, int64_t last_before,
                         int64_t active, int add) {
  return qt_mode_product(c, C, A, B, last_before, active, active, 1, add);
}

int qt_qr_orthogonal(qt_ctx* c) {
  if (!c) return fail(c, QT_ERR_ARG, "null context");
  QT_DEVICE(c);
  if (!c->prepared) return fail(c, QT_ERR_STATE, "qt_qr_orthogonal before qt_prepare");
  if (!c->have_psi) return fail(c, QT_ERR_STATE, "no wavefunction uploaded");
  const qt::Plan& P = c->plan;
  const auto& nd = P.nodes;
  double2* psi = c->buf[qt::B_PSI64];
  double2* scr = c->buf[qt::B_SCR];
  const int64_t cap = c->buf_elems[qt::B_SCR];
  int max_h = 0;
  for (const auto& g : nd) max_h = std::max(max_h, g.height);
  // per height: Q scratch, R, the task records and the parent's temporary copy
  for (int h = 0; h <= max_h; ++h) {
    std::vector<int> ids;
    for (int a = 0; a < (int)nd.size(); ++a)
      if (!nd[a].top() && nd[a].height == h) ids.push_back(a);
    if (ids.empty()) continue;
    std::vector<qt::QRTask> tasks;
    int64_t off = 0, tmp = 0;
    for (int a : ids) {
      const int64_t n = nd[a].dup(), m = nd[a].N / n;
      qt::QRTask t;
      t.A = psi + nd[a].off;
      t.Qs = scr + off;
      off += m * n;
      t.R = scr + off;
      off += n * n;
      t.m = (int)m;
      t.n = (int)n;
      tasks.push_back(t);
      tmp = std::max(tmp, nd[nd[a].parent].N);
    }
    const int64_t task_elems = ((int64_t)(tasks.size() * sizeof(qt::QRTask)) + 15) / 16;
    if (off + tmp + task_elems > cap)
      return fail(c, QT_ERR_ALLOC, "qt_qr_orthogonal: the chain scratch is too small for one height");
    double2* ptmp = scr + off;
    void* dtasks = scr + off + tmp;
    QT_CUDA(c, cudaMemcpyAsync(dtasks, tasks.data(), tasks.size() * sizeof(qt::QRTask), cudaMemcpyHostToDevice,
                               c->stream));
    QT_CUDA(c, qt::launch_house_qr(dtasks, (int)tasks.size(), c->stream));
    c->launches += 1;
    // R into the parents along the child index (siblings of one parent in turn)
    for (size_t i = 0; i < ids.size(); ++i) {
      const qt::NodeGeo& g = nd[ids[i]];
      const qt::NodeGeo& pg = nd[g.parent];
      qt::MPTask t;
      t.in = psi + pg.off;
      t.out = ptmp;
      t.h = tasks[i].R;
      t.alpha = make_double2(1.0, 0.0);
      t.before = (int)pg.before(g.child_idx);
      t.a_in = t.a_out = g.dup();
      t.after = (int)pg.after(g.child_idx);
      t.diag = 0;
      t.add = 0;
      QT_CUDA(c, qt::launch_single_mp(t, c->stream, nullptr));
      QT_CUDA(c, cudaMemcpyAsync(psi + pg.off, ptmp, pg.N * 16, cudaMemcpyDeviceToDevice, c->stream));
      c->launches += 1;
    }
    // the task records must outlive their copy
    QT_CUDA(c, cudaStreamSynchronize(c->stream));
  }
  c->swept = false;
  return QT_OK;
}

int qt_dev_alloc(qt_ctx* c, int64_t bytes, void** p) {
  if (!c || !p || bytes <= 0) return fail(c, QT_ERR_ARG, "qt_dev_alloc: bad argument");
  QT_DEVICE(c);
  cudaError_t e = dev_malloc(p, (size_t)bytes);
  if (e != cudaSuccess) return fail(c, QT_ERR_ALLOC, std::string("qt_dev_alloc: ") + cudaGetErrorString(e));
  return QT_OK;
}

int qt_dev_free(qt_ctx* c, void* p) {
  if (!c) return fail(c, QT_ERR_ARG, "null context");
  QT_DEVICE(c);
  QT_CUDA(c, cudaStreamSynchronize(c->stream));
  QT_CUDA(c, cudaFree(p));
  return QT_OK;
}

int qt_memcpy_h2d(qt_ctx* c, void* dst, const void* src, int64_t bytes) {
  if (!c || !dst || !src || bytes < 0) return fail(c, QT_ERR_ARG, "qt_memcpy_h2d: bad argument");
  QT_DEVICE(c);
  QT_CUDA(c, cudaMemcpyAsync(dst, src, (size_t)bytes, cudaMemcpyHostToDevice, c->stream));
  QT_CUDA(c, cudaStreamSynchronize(c->stream));
  return QT_OK;
}

int qt_memcpy_d2h(qt_ctx* c, void* dst, const void* src, int64_t bytes) {
  if (!c || !dst || !src || bytes < 0) return fail(c, QT_ERR_ARG, "qt_memcpy_d2h: bad argument");
  QT_DEVICE(c);
  QT_CUDA(c, cudaMemcpyAsync(dst, src, (size_t)bytes, cudaMemcpyDeviceToHost, c->stream));
  QT_CUDA(c, cudaStreamSynchronize(c->stream));
  return QT_OK;
}

int64_t qt_launch_count(const qt_ctx* c) { return c ? c->launches : -1; }

int qt_stage_count(const qt_ctx* c) { return (c && c->prepared) ? (int)c->plan.main_end : -1; }

int qt_stage_info(const qt_ctx* c, int i, int* kind, int64_t* tiles, double* flops, double* bytes) {
  if (!c || !c->prepared || i < 0 || i >= (int)c->plan.main_end) return QT_ERR_ARG;
  const auto& st = c->plan.stages[i];
  if (kind) *kind = st.kind;
  if (tiles)
    *tiles = st.kind == qt::ST_MP || st.kind == qt::ST_HP || st.kind == qt::ST_ACC || st.kind == qt::ST_MM
                 ? st.n_tiles
                 : st.n_tasks;
  if (flops) *flops = st.flops;
  if (bytes) *bytes = st.bytes;
  return QT_OK;
}

int qt_stage_launch(qt_ctx* c, int i) {
  if (!c) return fail(c, QT_ERR_ARG, "null context");
  if (!c->prepared || !c->have_psi) return fail(c, QT_ERR_STATE, "qt_stage_launch needs a prepared context and a wavefunction");
  if (i < 0 || i >= (int)c->plan.main_end) return fail(c, QT_ERR_ARG, "no such stage");
  QT_DEVICE(c);
  cudaError_t e = qt::launch_stage(c->plan.stages[i], c->tables, c->eps, c->plan.max_eig_d, c->prec,
                                   c->stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "qt_stage_launch");
  c->launches += kernels_in(c->plan, i, i + 1);
  return QT_OK;
}

int qt_rho_inverse_noalloc(qt_ctx* c, void* rhoinv, const void* rho, int n_mats, int d, double eps) {
  if (!c || !rhoinv || !rho) return fail(c, QT_ERR_ARG, "qt_rho_inverse_noalloc: null argument");
  if (n_mats < 1 || d < 1 || d > 112)
    return fail(c, QT_ERR_SHAPE, "qt_rho_inverse_noalloc: need n_mats >= 1 and 1 <= d <= 112");
  if (!(eps > 0) || !std::isfinite(eps)) return fail(c, QT_ERR_ARG, "qt_rho_inverse_noalloc: eps must be positive");
  const int64_t need = (int64_t)n_mats * d * d;
  if (need > qt::static_eig_capacity())
    return fail(c, QT_ERR_SHAPE,
                "qt_rho_inverse_noalloc: n_mats*d*d = " + std::to_string(need) +
                    " exceeds the static scratch of " + std::to_string(qt::static_eig_capacity()) +
                    " complex elements (8 MiB)");
  {
    // the kernel reads rho while other blocks write rhoinv: the ranges must not overlap at all
    const uintptr_t r0 = (uintptr_t)rho, w0 = (uintptr_t)rhoinv, bytes = (uintptr_t)need * 16;
    if (r0 < w0 + bytes && w0 < r0 + bytes)
      return fail(c, QT_ERR_ARG, "qt_rho_inverse_noalloc: the rho and rhoinv ranges overlap");
  }
  QT_DEVICE(c);
  cudaError_t e = qt::launch_rho_inverse_static((const double2*)rho, (double2*)rhoinv, n_mats, d, eps,
                                                c->stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "qt_rho_inverse_noalloc");
  c->launches += 1;
  return QT_OK;
}

int qt_probe_df64_peak(qt_ctx* c, double* tflops) {
  if (!c || !tflops) return fail(c, QT_ERR_ARG, "null argument");
  QT_DEVICE(c);
  double v = 0;
  cudaError_t e = qt::probe_df64_peak(c->stream, &v);
  if (e != cudaSuccess) return cuda_fail(c, e, "qt_probe_df64_peak");
  c->launches += 2;
  *tflops = v;
  return QT_OK;
}

int qt_probe_fp64_peak(qt_ctx* c, double* tflops) {
  if (!c || !tflops) return fail(c, QT_ERR_ARG, "null argument");
  QT_DEVICE(c);
  double v = 0;
  cudaError_t e = qt::probe_fp64_peak(c->stream, &v);
  if (e != cudaSuccess) return cuda_fail(c, e, "qt_probe_fp64_peak");
  c->launches += 2;
  *tflops = v;
  return QT_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// SCF / Krylov sweep (QT_PLAN_SCF): the scf() driver of QuTree
// (src/Applications/SCF.cpp:267-341) around the plan's per-node segments.
// ---------------------------------------------------------------------------
namespace {

using cd = double2;
constexpr double kLanczosBreakdown = 1e-12;  // residual norm / |T| below which the space is invariant

int run_stages(qt_ctx* c, int64_t b, int64_t e) {
  const Plan& P = c->plan;
  for (int64_t i = b; i < e; ++i) {
    cudaError_t err = qt::launch_stage(P.stages[i], c->tables, c->eps, P.max_eig_d, c->prec, c->stream);
    if (err != cudaSuccess) return cuda_fail(c, err, P.stages[i].name);
  }
  c->launches += kernels_in(P, b, e);
  return QT_OK;
}

inline cd cmk(double x, double y) { return make_double2(x, y); }
inline cd cmulh(cd a, cd b) { return cmk(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }
inline cd cconj(cd a) { return cmk(a.x, -a.y); }

// Eigen-decomposition of the symmetric tridiagonal Lanczos matrix (size <= 32)
// by cyclic Jacobi rotations; eigenvalues ascending, U(:, k) the eigenvectors.
void tridiag_eigh(const std::vector<double>& alpha, const std::vector<double>& beta, int m,
                  std::vector<double>& E, std::vector<double>& U) {
  std::vector<double> A(m * m, 0.0);
  U.assign(m * m, 0.0);
  for (int i = 0; i < m; ++i) {
    A[i + m * i] = alpha[i];
    U[i + m * i] = 1.0;
    if (i + 1 < m) A[i + 1 + m * i] = A[i + m * (i + 1)] = beta[i];
  }
  for (int sweep = 0; sweep < 100; ++sweep) {
    double off = 0.0, tot = 0.0;
    for (int j = 0; j < m; ++j)
      for (int i = 0; i < m; ++i) {
        tot += A[i + m * j] * A[i + m * j];
        if (i != j) off += A[i + m * j] * A[i + m * j];
      }
    if (off <= 1e-32 * tot || off == 0.0) break;
    for (int p = 0; p < m; ++p)
      for (int q = p + 1; q < m; ++q) {
        const double apq = A[p + m * q];
        if (apq == 0.0) continue;
        const double theta = (A[q + m * q] - A[p + m * p]) / (2.0 * apq);
        const double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
        const double cs = 1.0 / std::sqrt(t * t + 1.0), sn = t * cs;
        for (int k = 0; k < m; ++k) {  // columns p, q
          const double akp = A[k + m * p], akq = A[k + m * q];
          A[k + m * p] = cs * akp - sn * akq;
          A[k + m * q] = sn * akp + cs * akq;
        }
        for (int k = 0; k < m; ++k) {  // rows p, q
          const double apk = A[p + m * k], aqk = A[q + m * k];
          A[p + m * k] = cs * apk - sn * aqk;
          A[q + m * k] = sn * apk + cs * aqk;
        }
        for (int k = 0; k < m; ++k) {
          const double ukp = U[k + m * p], ukq = U[k + m * q];
          U[k + m * p] = cs * ukp - sn * ukq;
          U[k + m * q] = sn * ukp + cs * ukq;
        }
      }
  }
  std::vector<int> idx(m);
  for (int i = 0; i < m; ++i) idx[i] = i;
  std::sort(idx.begin(), idx.end(), [&](int x, int y) { return A[x + m * x] < A[y + m * y]; });
  std::vector<double> U2(m * m);
  E.assign(m, 0.0);
  for (int k = 0; k < m; ++k) {
    E[k] = A[idx[k] + m * idx[k]];
    for (int i = 0; i < m; ++i) U2[i + m * k] = U[i + m * idx[k]];
  }
  U.swap(U2);
}

// S = R^dag R with R upper triangular (complex Cholesky); false when S is not
// numerically positive definite (smallest pivot <= tol * largest)
bool cholesky_upper(const std::vector<cd>& S, int d, std::vector<cd>& R, double tol) {
  R.assign(d * d, cmk(0, 0));
  double pmax = 0.0, pmin = 1e300;
  for (int j = 0; j < d; ++j) {
    // R(j, j) = sqrt(S(j,j) - sum_k |R(k,j)|^2)
    double s = S[j + d * j].x;
    for (int k = 0; k < j; ++k) s -= R[k + d * j].x * R[k + d * j].x + R[k + d * j].y * R[k + d * j].y;
    if (!(s > 0.0) || !std::isfinite(s)) return false;
    const double rjj = std::sqrt(s);
    R[j + d * j] = cmk(rjj, 0);
    pmax = std::max(pmax, rjj);
    pmin = std::min(pmin, rjj);
    for (int i = j + 1; i < d; ++i) {
      // R(j, i) = (S(j, i) - sum_k conj(R(k, j)) R(k, i)) / R(j, j)
      cd v = S[j + d * i];
      for (int k = 0; k < j; ++k) {
        const cd p = cmulh(cconj(R[k + d * j]), R[k + d * i]);
        v.x -= p.x;
        v.y -= p.y;
      }
      R[j + d * i] = cmk(v.x / rjj, v.y / rjj);
    }
  }
  return pmin > tol * pmax;
}

// h = (R^-1)^T for an upper-triangular R, so that Y x_mode h = Y R^-1
void inv_upper_transposed(const std::vector<cd>& R, int d, std::vector<cd>& h) {
  std::vector<cd> X(d * d, cmk(0, 0));  // X = R^-1, upper triangular
  for (int j = 0; j < d; ++j) {
    const double den = R[j + d * j].x * R[j + d * j].x + R[j + d * j].y * R[j + d * j].y;
    X[j + d * j] = cmk(R[j + d * j].x / den, -R[j + d * j].y / den);
    for (int i = j - 1; i >= 0; --i) {
      cd v = cmk(0, 0);
      for (int k = i + 1; k <= j; ++k) {
        const cd p = cmulh(R[i + d * k], X[k + d * j]);
        v.x += p.x;
        v.y += p.y;
      }
      const cd rii = R[i + d * i];
      const double dd = rii.x * rii.x + rii.y * rii.y;
      const cd inv = cmk(rii.x / dd, -rii.y / dd);
      const cd q = cmulh(v, inv);
      X[i + d * j] = cmk(-q.x, -q.y);
    }
  }
  h.assign(d * d, cmk(0, 0));
  for (int a = 0; a < d; ++a)
    for (int b = 0; b < d; ++b) h[b + d * a] = X[a + d * b];
}

// Thin Q of the m x d column-major matrix M (m >= d) by Householder
// reflections with LAPACK's convention (zgeqrf / zungqr: beta = -sign(Re alpha) |x|)
void householder_thin_q(std::vector<cd>& M, int64_t m, int d) {
  std::vector<cd> tau(d, cmk(0, 0));
  for (int k = 0; k < d; ++k) {
    cd* x = &M[(size_t)k * m + k];
    const int64_t len = m - k;
    double xn2 = 0.0;
    for (int64_t i = 1; i < len; ++i) xn2 += x[i].x * x[i].x + x[i].y * x[i].y;
    const cd alpha = x[0];
    if (xn2 == 0.0 && alpha.y == 0.0) {
      tau[k] = cmk(0, 0);
    } else {
      double beta = std::sqrt(alpha.x * alpha.x + alpha.y * alpha.y + xn2);
      if (alpha.x >= 0.0) beta = -beta;
      tau[k] = cmk((beta - alpha.x) / beta, -alpha.y / beta);
      const cd den = cmk(alpha.x - beta, alpha.y);
      const double dd = den.x * den.x + den.y * den.y;
      const cd inv = cmk(den.x / dd, -den.y / dd);
      for (int64_t i = 1; i < len; ++i) x[i] = cmulh(x[i], inv);
      x[0] = cmk(beta, 0);
    }
    // apply H^H = I - conj(tau) v v^H to the columns right of k (v(0) = 1)
    const cd tc = cconj(tau[k]);
    for (int j = k + 1; j < d; ++j) {
      cd* y = &M[(size_t)j * m + k];
      cd w = y[0];
      for (int64_t i = 1; i < len; ++i) {
        const cd p = cmulh(cconj(x[i]), y[i]);
        w.x += p.x;
        w.y += p.y;
      }
      const cd f = cmulh(tc, w);
      y[0].x -= f.x;
      y[0].y -= f.y;
      for (int64_t i = 1; i < len; ++i) {
        const cd p = cmulh(x[i], f);
        y[i].x -= p.x;
        y[i].y -= p.y;
      }
    }
  }
  // Q = H_0 H_1 ... H_{d-1} applied to the first d columns of the identity
  std::vector<cd> Q((size_t)m * d, cmk(0, 0));
  for (int j = 0; j < d; ++j) Q[(size_t)j * m + j] = cmk(1, 0);
  for (int k = d - 1; k >= 0; --k) {
    const cd* v = &M[(size_t)k * m + k];
    const int64_t len = m - k;
    for (int j = k; j < d; ++j) {
      cd* y = &Q[(size_t)j * m + k];
      cd w = y[0];
      for (int64_t i = 1; i < len; ++i) {
        const cd p = cmulh(cconj(v[i]), y[i]);
        w.x += p.x;
        w.y += p.y;
      }
      const cd f = cmulh(tau[k], w);
      y[0].x -= f.x;
      y[0].y -= f.y;
      for (int64_t i = 1; i < len; ++i) {
        const cd p = cmulh(v[i], f);
        y[i].x -= p.x;
        y[i].y -= p.y;
      }
    }
  }
  M.swap(Q);
}

// scf_sweep: depth first from the top, back to the node after each child
void sweep_order(const std::vector<qt::NodeGeo>& nd, int a, std::vector<int>& out) {
  out.push_back(a);
  for (int c : nd[a].children) {
    sweep_order(nd, c, out);
    out.push_back(a);
  }
}

struct DevFree {
  void* p = nullptr;
  ~DevFree() {
    if (p) cudaFree(p);
  }
};

}  // namespace

int qt_scf(qt_ctx* c, int n_iter, int n_krylov, int n_itp, double beta, double* ritz, int64_t ritz_capacity,
           int64_t* ritz_count) {
  if (!c) return fail(c, QT_ERR_ARG, "null context");
  if (!c->prepared || !c->have_psi) return fail(c, QT_ERR_STATE, "qt_scf needs qt_prepare and a wavefunction");
  const Plan& P = c->plan;
  if (!P.scf) return fail(c, QT_ERR_STATE, "plan prepared without QT_PLAN_SCF");
  if (P.tops.size() != 1) return fail(c, QT_ERR_SHAPE, "qt_scf sweeps one tree");
  if (n_iter < 0 || n_krylov < 1 || n_krylov > qt::kLinCombMax - 2 || n_itp < 0)
    return fail(c, QT_ERR_ARG, "qt_scf: n_iter >= 0, 1 <= n_krylov <= 30, n_itp >= 0");
  const std::vector<qt::NodeGeo>& nd = P.nodes;
  std::vector<int> order;
  sweep_order(nd, P.tops[0], order);
  const int64_t solves = (int64_t)n_iter * (int64_t)order.size();
  if (ritz && ritz_capacity < solves) return fail(c, QT_ERR_ARG, "qt_scf: ritz buffer too small");
  if (ritz_count) *ritz_count = 0;
  QT_DEVICE(c);
  int64_t maxN = 16;
  int maxd = 1;
  for (const auto& g : nd) {
    maxN = std::max(maxN, g.N);
    for (int x : g.shape) maxd = std::max(maxd, x);
  }
  const int64_t vstride = (maxN + 15) / 16 * 16, mstride = (int64_t)maxd * maxd;
  // vectors V_0..V_{K-1}, W, Y, T, U; matrices S, H, R; dot scratch; hole-product partial tiles
  const int64_t ws_elems = 64 * mstride;
  const int64_t total = (n_krylov + 4) * vstride + 3 * mstride + 512 + ws_elems;
  DevFree work;
  {
    cudaError_t e = dev_malloc(&work.p, total * sizeof(cd));
    if (e != cudaSuccess) return fail(c, QT_ERR_ALLOC, std::string("qt_scf: work allocation failed: ") + cudaGetErrorString(e));
  }
  cd* base = (cd*)work.p;
  auto V = [&](int l) { return base + (int64_t)l * vstride; };
  cd* W = V(n_krylov);
  cd* Y = V(n_krylov + 1);
  cd* T = V(n_krylov + 2);
  cd* U = V(n_krylov + 3);  // complex128 copy of H v (double-float plans)
  cd* dS = base + (n_krylov + 4) * vstride;
  cd* dH = dS + mstride;
  cd* dR = dH + mstride;
  cd* dscal = dR + mstride;
  cd* hpws = dscal + 512;
  // the driver works on the complex128 wavefunction; with double-float
  // arithmetic the plan's stages read B_PSI, refreshed node by node
  const bool df = c->prec >= 1;
  cd* psi = c->buf[qt::B_PSI64];
  cd* psi_ar = c->buf[qt::B_PSI];
  cd* kin = c->buf[qt::B_KRY] + P.kry_in;
  cd* kout = c->buf[qt::B_KRY] + P.kry_out;
  cd* hv = df ? U : kout;  // H v in complex128
  auto to_arith = [&](cd* dst, const cd* src, int64_t n) -> int {
    cudaError_t e = qt::launch_convert(dst, src, n, 0, c->stream);
    if (e != cudaSuccess) return cuda_fail(c, e, "qt_scf convert");
    c->launches += 1;
    return QT_OK;
  };
  auto dot = [&](const cd* a, const cd* b, int64_t n, cd& out) -> int {
    cudaError_t e = qt::launch_dot(a, b, n, dscal, c->stream);
    if (e != cudaSuccess) return cuda_fail(c, e, "qt_scf dot");
    QT_CUDA(c, cudaMemcpyAsync(&out, dscal, sizeof(cd), cudaMemcpyDeviceToHost, c->stream));
    QT_CUDA(c, cudaStreamSynchronize(c->stream));
    c->launches += 2;
    return QT_OK;
  };
  auto lincomb = [&](cd* out, std::initializer_list<std::pair<const cd*, cd>> terms, int64_t n) -> int {
    qt::LinComb lc;
    lc.count = 0;
    for (auto& t : terms) {
      lc.v[lc.count] = t.first;
      lc.c[lc.count] = t.second;
      ++lc.count;
    }
    cudaError_t e = qt::launch_lincomb(out, lc, n, c->stream);
    if (e != cudaSuccess) return cuda_fail(c, e, "qt_scf lincomb");
    c->launches += 1;
    return QT_OK;
  };
  auto hole = [&](const cd* A, const cd* B, const qt::NodeGeo& g, int mode, cd* S) -> int {
    qt::HPTask t;
    t.A = A;
    t.B = B;
    t.S = S;
    t.before = (int)g.before(mode);
    t.a = g.shape[mode];
    t.after = (int)g.after(mode);
    t.aB = 0;
    t.splits = 1;
    t.kchunk = 0;
    t.ws = 0;
    t.rows = t.cols = 4;
    cudaError_t e = qt::launch_hp_split(t, hpws, ws_elems, c->stream);
    if (e != cudaSuccess) return cuda_fail(c, e, "qt_scf hole product");
    c->launches += 1;
    return QT_OK;
  };
  auto mode_product = [&](const cd* h, const cd* in, cd* out, const qt::NodeGeo& g, int mode) -> int {
    qt::MPTask t;
    t.in = in;
    t.out = out;
    t.h = h;
    t.alpha = cmk(1, 0);
    t.before = (int)g.before(mode);
    t.a_in = t.a_out = g.shape[mode];
    t.after = (int)g.after(mode);
    t.diag = 0;
    t.add = 0;
    cudaError_t e = qt::launch_single_mp(t, c->stream, nullptr);
    if (e != cudaSuccess) return cuda_fail(c, e, "qt_scf mode product");
    c->launches += 1;
    return QT_OK;
  };
  int rc;
  if (df && (rc = to_arith(psi_ar, psi, P.psi_packed)) != QT_OK) return rc;
  // initial build: buildSCF(node, parent) for every non-top node, bottom-up
  for (size_t a = 0; a < nd.size(); ++a)
    if (!nd[a].top() && (rc = run_stages(c, P.scf_up_b[a], P.scf_up_e[a])) != QT_OK) return rc;
  int64_t nritz = 0;
  std::vector<cd> hS, hR, hR2, hh;
  for (int it = 0; it < n_iter; ++it) {
    for (size_t i = 0; i < order.size(); ++i) {
      const int a = order[i];
      const qt::NodeGeo& g = nd[a];
      const int64_t N = g.N;
      cd* pa = psi + g.aoff;
      int size = (int)std::min<int64_t>(n_krylov, N);
      // Lanczos on the effective Hamiltonian (solveKrylovSpace)
      std::vector<double> al, be;
      cd s;
      if ((rc = dot(pa, pa, N, s)) != QT_OK) return rc;
      if (!(s.x > 0.0) || !std::isfinite(s.x)) return fail(c, QT_ERR_NUMERIC, "qt_scf: zero or non-finite node tensor");
      if ((rc = lincomb(V(0), {{pa, cmk(1.0 / std::sqrt(s.x), 0)}}, N)) != QT_OK) return rc;
      for (int l = 0; l < size; ++l) {
        if (df) {
          if ((rc = to_arith(kin, V(l), N)) != QT_OK) return rc;
        } else {
          QT_CUDA(c, cudaMemcpyAsync(kin, V(l), N * sizeof(cd), cudaMemcpyDeviceToDevice, c->stream));
        }
        if ((rc = run_stages(c, P.scf_apply_b[a], P.scf_apply_e[a])) != QT_OK) return rc;
        if (df) {
          cudaError_t e = qt::launch_convert(U, kout, N, 1, c->stream);
          if (e != cudaSuccess) return cuda_fail(c, e, "qt_scf convert");
          c->launches += 1;
        }
        if ((rc = dot(V(l), hv, N, s)) != QT_OK) return rc;
        if (!std::isfinite(s.x)) return fail(c, QT_ERR_NUMERIC, "qt_scf: non-finite <v|H|v>");
        al.push_back(s.x);
        if (l + 1 == size) break;
        if (l == 0)
          rc = lincomb(W, {{hv, cmk(1, 0)}, {V(0), cmk(-al[0], 0)}}, N);
        else
          rc = lincomb(W, {{hv, cmk(1, 0)}, {V(l), cmk(-al[l], 0)}, {V(l - 1), cmk(-be[l - 1], 0)}}, N);
        if (rc != QT_OK) return rc;
        if ((rc = dot(W, W, N, s)) != QT_OK) return rc;
        const double nrm = std::sqrt(std::max(s.x, 0.0));
        if (!std::isfinite(nrm)) return fail(c, QT_ERR_NUMERIC, "qt_scf: non-finite Lanczos residual");
        // an invariant subspace: the residual is rounding noise (the reference
        // divides by it); the Lanczos space ends here
        double scale = 0.0;
        for (double x : al) scale = std::max(scale, std::fabs(x));
        for (double x : be) scale = std::max(scale, x);
        if (nrm <= kLanczosBreakdown * scale) {
          size = l + 1;
          break;
        }
        be.push_back(nrm);
        if ((rc = lincomb(V(l + 1), {{W, cmk(1.0 / nrm, 0)}}, N)) != QT_OK) return rc;
      }
      std::vector<double> E, U;
      tridiag_eigh(al, be, size, E, U);
      if (ritz) ritz[nritz] = E[0];
      ++nritz;
      // imaginaryTimePropagation (the k = 0 term enters twice, SCF.cpp:208-214) or the Ritz vector
      qt::LinComb lc;
      lc.count = size;
      for (int l = 0; l < size; ++l) {
        lc.v[l] = V(l);
        double cl;
        if (it < n_itp) {
          cl = U[l] * U[0];
          for (int k = 0; k < size; ++k) cl += U[l + size * k] * std::exp(-beta * (E[k] - E[0])) * U[size * k];
        } else {
          cl = U[l];
        }
        lc.c[l] = cmk(cl, 0);
      }
      {
        cudaError_t e = qt::launch_lincomb(Y, lc, N, c->stream);
        if (e != cudaSuccess) return cuda_fail(c, e, "qt_scf lincomb");
        c->launches += 1;
      }
      if (it < n_itp) {
        if ((rc = dot(Y, Y, N, s)) != QT_OK) return rc;
        if ((rc = lincomb(Y, {{Y, cmk(1.0 / std::sqrt(s.x), 0)}}, N)) != QT_OK) return rc;
      }
      // isometrize toward the next node: Cholesky-QR twice, Householder when
      // the Gram matrix is near singular
      const int nxt = i + 1 < order.size() ? order[i + 1] : -1;
      int out_idx = g.last();
      for (size_t k = 0; k < g.children.size(); ++k)
        if (g.children[k] == nxt) out_idx = (int)k;
      const int d = g.shape[out_idx];
      bool chol_ok = true;
      const cd* src = Y;
      for (int pass = 0; pass < 2 && chol_ok; ++pass) {
        if ((rc = hole(src, src, g, out_idx, dS)) != QT_OK) return rc;
        hS.resize((size_t)d * d);
        QT_CUDA(c, cudaMemcpyAsync(hS.data(), dS, (size_t)d * d * sizeof(cd), cudaMemcpyDeviceToHost, c->stream));
        QT_CUDA(c, cudaStreamSynchronize(c->stream));
        if (!cholesky_upper(hS, d, hR, 1e-6)) {
          chol_ok = false;
          break;
        }
        inv_upper_transposed(hR, d, hh);
        QT_CUDA(c, cudaMemcpyAsync(dH, hh.data(), (size_t)d * d * sizeof(cd), cudaMemcpyHostToDevice, c->stream));
        if ((rc = mode_product(dH, src, pass == 0 ? T : pa, g, out_idx)) != QT_OK) return rc;
        src = T;
      }
      if (!chol_ok) {
        const int64_t bef = g.before(out_idx), aft = g.after(out_idx), m = bef * aft;
        if (m < d) return fail(c, QT_ERR_SHAPE, "qt_scf: node dimension below its bond");
        std::vector<cd> hy(N), M((size_t)m * d);
        QT_CUDA(c, cudaMemcpyAsync(hy.data(), Y, N * sizeof(cd), cudaMemcpyDeviceToHost, c->stream));
        QT_CUDA(c, cudaStreamSynchronize(c->stream));
        for (int64_t af = 0; af < aft; ++af)  // toMatrix(Y, mode): row = bef + aft * before
          for (int x = 0; x < d; ++x)
            for (int64_t bf = 0; bf < bef; ++bf) M[(size_t)x * m + bf + af * bef] = hy[bf + bef * (x + (int64_t)d * af)];
        householder_thin_q(M, m, d);
        for (int64_t af = 0; af < aft; ++af)
          for (int x = 0; x < d; ++x)
            for (int64_t bf = 0; bf < bef; ++bf) hy[bf + bef * (x + (int64_t)d * af)] = M[(size_t)x * m + bf + af * bef];
        QT_CUDA(c, cudaMemcpyAsync(pa, hy.data(), N * sizeof(cd), cudaMemcpyHostToDevice, c->stream));
        QT_CUDA(c, cudaStreamSynchronize(c->stream));
      }
      if (nxt < 0) break;
      // r = <Q|Y> over out_idx, multiplied into the next node; rebuild toward it
      if ((rc = hole(pa, Y, g, out_idx, dR)) != QT_OK) return rc;
      const qt::NodeGeo& gn = nd[nxt];
      int in_idx = gn.last();
      for (size_t k = 0; k < gn.children.size(); ++k)
        if (gn.children[k] == a) in_idx = (int)k;
      cd* pn = psi + gn.aoff;
      if ((rc = mode_product(dR, pn, T, gn, in_idx)) != QT_OK) return rc;
      QT_CUDA(c, cudaMemcpyAsync(pn, T, gn.N * sizeof(cd), cudaMemcpyDeviceToDevice, c->stream));
      if (df) {
        if ((rc = to_arith(psi_ar + g.aoff, pa, N)) != QT_OK) return rc;
        if ((rc = to_arith(psi_ar + gn.aoff, pn, gn.N)) != QT_OK) return rc;
      }
      const bool up = !g.top() && g.parent == nxt;
      if (up)
        rc = run_stages(c, P.scf_up_b[a], P.scf_up_e[a]);
      else
        rc = run_stages(c, P.scf_down_b[nxt], P.scf_down_e[nxt]);
      if (rc != QT_OK) return rc;
    }
  }
  QT_CUDA(c, cudaStreamSynchronize(c->stream));
  if (ritz_count) *ritz_count = nritz;
  c->swept = false;
  c->built = false;
  return QT_OK;
}
