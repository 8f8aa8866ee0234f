// gpu_sweep_shim.cpp -- the QuTree-side binding of the integration guide,
// compiled by g++ against include/qtgpu.h and linked against libqtgpu.so,
// around minimal stand-ins for QuTree's types (qutree_standins.h).  The
// class between the shim markers is the documented one, character for
// character (a CPU test checks that).
//
// main(): reads a problem written by tests/test_cpp_boundary.py (tree,
// leaf operators, SOP terms, packed wavefunction), runs one
// GpuSweep::derivative -- the drop-in for QuTree's Derivative()
// (src/TreeClasses/HamiltonianRepresentation.cpp:74-81) -- and writes dPsi
// and <Phi_top|H|Phi_top>, <Phi_top|Phi_top>.
//
// usage: gpu_sweep_shim <problem file> <result file> <plan flavour>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <iostream>
#include <string>

#include "qtgpu.h"
#include "qutree_standins.h"

// ---- shim begin ----
class GpuSweep {
 public:
  GpuSweep(const Hamiltonian& H, const Tree& tree, int device = 0,
           int flavour = QT_PLAN_COMPRESSED | QT_PREC_DF64) {
    check(qt_ctx_create(&ctx_, device));
    std::vector<int> order, dims, parent, child, leaf;
    for (const Node& n : tree) {
      const TensorShape& s = n.shape();
      order.push_back((int)s.order());
      for (size_t k = 0; k < s.order(); ++k) dims.push_back((int)s[k]);
      parent.push_back(n.isToplayer() ? -1 : (int)n.parent().address());
      child.push_back(n.isToplayer() ? -1 : (int)n.childIdx());
      leaf.push_back(n.isBottomlayer() ? (int)n.getLeaf().mode() : -1);
    }
    check(qt_tree_upload(ctx_, (int)order.size(), order.data(), dims.data(),
                         parent.data(), child.data(), leaf.data()));
    // operator table: materialise every leaf operator as a dense p x p
    // matrix by applying it to the unit vectors of its leaf
    std::vector<int> kind, dim, ptr{0}, tmode, top;
    std::vector<int64_t> off;
    std::vector<std::complex<double>> data, coeff;
    for (size_t l = 0; l < H.size(); ++l) {
      const MLOcd& M = H[l];
      for (size_t k = 0; k < M.size(); ++k) {
        const Leaf& leafk = tree.getLeaf(M.targetLeaves()[k]);
        size_t p = leafk.dim();
        Tensorcd unit({p, p});
        for (size_t i = 0; i < p; ++i) unit(i, i) = 1.;
        Tensorcd hu({p, p});
        M[k]->apply(leafk.interface(), hu, unit);        // columns = h e_i
        kind.push_back(QT_OP_DENSE); dim.push_back((int)p);
        off.push_back((int64_t)data.size());
        for (size_t i = 0; i < p * p; ++i) data.push_back(hu(i));
        tmode.push_back((int)M.targetLeaves()[k]);
        top.push_back((int)kind.size() - 1);
      }
      ptr.push_back((int)tmode.size());
      coeff.push_back(H.coeff(l));
    }
    check(qt_sop_upload(ctx_, (int)kind.size(), kind.data(), dim.data(), off.data(),
                        (const double*)data.data(), (int)H.size(),
                        (const double*)coeff.data(), ptr.data(), tmode.data(), top.data()));
    check(qt_prepare(ctx_, flavour));
    packed_.resize(qt_psi_size(ctx_));
  }
  ~GpuSweep() { qt_ctx_destroy(ctx_); }

  // drop-in for Derivative(dPsi, hRep, time, Psi, H, tree, phase)
  void derivative(Wavefunction& dPsi, const Wavefunction& Psi, const Tree& tree,
                  std::complex<double> phase = 1.) {
    size_t o = 0;
    for (const Node& n : tree) {
      const Tensorcd& phi = Psi[n];
      std::copy(&phi[0], &phi[0] + phi.shape().totalDimension(), &packed_[o]);
      o += phi.shape().totalDimension();
    }
    check(qt_psi_upload(ctx_, (const double*)packed_.data()));
    check(qt_derivative(ctx_, phase.real(), phase.imag()));
    check(qt_dpsi_download(ctx_, (double*)packed_.data()));
    o = 0;
    for (const Node& n : tree) {
      Tensorcd& d = dPsi[n];
      std::copy(&packed_[o], &packed_[o] + d.shape().totalDimension(), &d[0]);
      o += d.shape().totalDimension();
    }
  }

  // Expectation(hRep, Psi, H, tree): {<Phi_top|H Phi_top>, <Phi_top|Phi_top>}
  void energy(std::complex<double>& h00, std::complex<double>& s00) {
    double e[4];
    check(qt_energy(ctx_, e));
    h00 = {e[0], e[1]};
    s00 = {e[2], e[3]};
  }

 private:
  void check(int rc) {
    if (rc != QT_OK) { std::cerr << qt_last_error(ctx_) << "\n"; exit(1); }  // QuTree's convention
  }
  qt_ctx* ctx_ = nullptr;
  std::vector<std::complex<double>> packed_;
};
// ---- shim end ----

namespace {

struct Reader {
  FILE* f;
  template <typename T>
  T get() {
    T v{};
    if (std::fread(&v, sizeof(T), 1, f) != 1) {
      std::cerr << "problem file truncated\n";
      exit(2);
    }
    return v;
  }
};

}  // namespace

int main(int argc, char** argv) {
  if (argc != 4) {
    std::cerr << "usage: gpu_sweep_shim <problem> <result> <flavour>\n";
    return 2;
  }
  FILE* f = std::fopen(argv[1], "rb");
  if (!f) {
    std::cerr << "cannot open " << argv[1] << "\n";
    return 2;
  }
  Reader r{f};
  // tree: per node order, dims, parent, child index, leaf mode; leaves: dims
  const int n_nodes = r.get<int32_t>();
  std::vector<Node> nodes;
  for (int a = 0; a < n_nodes; ++a) {
    const int order = r.get<int32_t>();
    std::vector<size_t> dims;
    for (int k = 0; k < order; ++k) dims.push_back((size_t)r.get<int32_t>());
    const int parent = r.get<int32_t>(), child = r.get<int32_t>(), leaf = r.get<int32_t>();
    nodes.emplace_back((size_t)a, TensorShape(dims), parent, child, leaf);
  }
  const int n_leaves = r.get<int32_t>();
  std::vector<Leaf> leaves;
  for (int m = 0; m < n_leaves; ++m) leaves.emplace_back((size_t)r.get<int32_t>(), (size_t)m);
  Tree tree(std::move(nodes), std::move(leaves));
  // operators: kind (0 dense, 1 diagonal), p, values
  const int n_ops = r.get<int32_t>();
  std::vector<std::shared_ptr<LeafOperatorcd>> ops;
  for (int i = 0; i < n_ops; ++i) {
    const int kind = r.get<int32_t>(), p = r.get<int32_t>();
    std::vector<cd> m(kind == 0 ? (size_t)p * p : (size_t)p);
    for (auto& v : m) {
      const double re = r.get<double>(), im = r.get<double>();
      v = cd(re, im);
    }
    ops.push_back(std::make_shared<LeafOperatorcd>((size_t)p, kind == 1, std::move(m)));
  }
  // terms: coefficient, factors (mode, operator) in MLO order
  Hamiltonian H;
  const int n_terms = r.get<int32_t>();
  for (int l = 0; l < n_terms; ++l) {
    const double cre = r.get<double>(), cim = r.get<double>();
    const int nf = r.get<int32_t>();
    MLOcd M;
    for (int k = 0; k < nf; ++k) {
      const int mode = r.get<int32_t>(), op = r.get<int32_t>();
      M.push_back(ops[(size_t)op], (size_t)mode);
    }
    H.push_back(M, cd(cre, cim));
  }
  Wavefunction Psi(tree), dPsi(tree);
  for (const Node& n : tree) {
    Tensorcd& phi = Psi[n];
    for (size_t i = 0; i < n.shape().totalDimension(); ++i) {
      const double re = r.get<double>(), im = r.get<double>();
      phi[i] = cd(re, im);
    }
  }
  std::fclose(f);

  GpuSweep gpu(H, tree, 0, std::atoi(argv[3]));
  gpu.derivative(dPsi, Psi, tree);
  cd h00, s00;
  gpu.energy(h00, s00);

  FILE* o = std::fopen(argv[2], "wb");
  if (!o) {
    std::cerr << "cannot open " << argv[2] << "\n";
    return 2;
  }
  const double e[4] = {h00.real(), h00.imag(), s00.real(), s00.imag()};
  bool ok = std::fwrite(e, sizeof(double), 4, o) == 4;
  for (const Node& n : tree) {
    const Tensorcd& d = dPsi[n];
    ok = ok && std::fwrite(&d[0], sizeof(cd), n.shape().totalDimension(), o) == n.shape().totalDimension();
  }
  ok = (std::fclose(o) == 0) && ok;
  return ok ? 0 : 3;
}
