// qt_plan.cpp -- host planner of the H.Psi sweep.
//
// Turns (tree, SOP) into a fixed list of batched GPU stages, executed in
// order for every sweep (and captured once as a CUDA graph):
//
//   1. density matrices, top-down by depth
//      (TreeFunctions::contraction(Rho, Psi, tree, true),
//       include/TreeClasses/MatrixTreeFunctions_Implementation.h:59-127)
//   2. regularised inverses of all density matrices
//      (SpectralDecompositionTree::calculate / invert,
//       src/TreeClasses/SpectralDecompositionTree.cpp:30-48)
//   3. represent, bottom-up by height
//      (TreeFunctions::represent,
//       include/TreeClasses/SparseMatrixTreeFunctions_Implementation.h:17-78)
//   4. mean fields, top-down by depth
//      (TreeFunctions::contraction / contractionLayer, same file :144-203)
//   5. Apply at every node (src/TreeClasses/HamiltonianRepresentation.cpp:6-43)
//   6. projector, inverse density and -i*phase (LayerDerivative, :53-72) and
//      the top-node expectation (Expectation, :45-51).
//
// Every represent / mean-field / apply step of the reference is a "chain":
// an input node tensor, up to a few mode products (or diagonal leaf
// operators), and a final hole product or last-mode accumulation.  All
// chains of one tree level run in the same launches: the chains' k-th mode
// products form one stage, their final contractions the next.
//
// Flavour QT_PLAN_REFERENCE keeps one chain per (SOP term, node), exactly the
// reference's call sequence.  Flavour QT_PLAN_GROUPED gives terms whose
// restriction to a node's subtree (represent, Apply) or to its complement
// (mean field) coincide one shared matrix and one chain: the reference
// computes the same matrix once per term; here it is computed once.  In
// Apply, terms with the same inside part share the chain and their mean
// fields are summed first (sum_l c_l H_l) x_last X, which is linear algebra
// on the same products.
#include <algorithm>
#include <cmath>
#include <map>
#include <set>
#include <stdexcept>
#include <tuple>

#include "qt_internal.h"

namespace qt {
namespace {

constexpr int kMpTile = 256;  // slots per mode-product tile: (b, four consecutive j, c), one per thread
constexpr int kAccRows = 64, kAccCols = 16;
constexpr int64_t kAlign = 16;  // elements (256 bytes)

int64_t align_up(int64_t x) { return (x + kAlign - 1) / kAlign * kAlign; }

double2 c2(double r, double i) {
  double2 v;
  v.x = r;
  v.y = i;
  return v;
}

struct COp {
  int kind;  // 0 mode product, 1 diagonal leaf operator
  int mode;
  Ref mat;
  double2 alpha;
};

struct Item {
  int node;  // geometry of the chain's tensors
  Ref in;
  std::vector<COp> ops;
  int fin;  // 0: hole product into S over hp_mode; 1: accumulate into hphi
  Ref S;
  int hp_mode = 0;
  int acc_node = -1;
  Ref accH;  // buf -1: identity
};

class Builder {
 public:
  Builder(Plan& P, const std::vector<NodeGeo>& nodes, const OpTable& ops, const SopDesc& sop,
          int flavour, int prec, int64_t budget)
      : P(P), nd(P.nodes), ops(ops), sop(sop), grouped(flavour == 1), compressed(flavour == 2),
        budget(budget) {
    if (flavour < 0 || flavour > 2) throw std::runtime_error("unknown plan flavour");
    P.nodes = nodes;
    P.prec = prec;
  }

  void set_scf(bool on) { scf = on; }
  void set_cdvr(const CdvrDesc* d) { cdvr = d; }

  void run() {
    geometry();
    activity();
    layout();
    if (P.prec >= 1) {
      int64_t c0 = (int64_t)P.cvt.size(), t0 = (int64_t)P.cvt_tiles.size();
      add_cvt(Ref{B_PSI64, 0}, Ref{B_PSI, 0}, P.psi_packed, 0);
      emit_stage(ST_CVT, c0, (int64_t)P.cvt.size(), t0, (int64_t)P.cvt_tiles.size(), "psi-in");
    }
    stage_density();
    stage_inverse();
    if (scf && !compressed) throw std::runtime_error("the SCF sweep needs the compressed plan");
    if (compressed) {
      comp_layout();
      comp_represent();
      comp_meanfield();
      if (P.want_grad) comp_environment();
      P.apply_begin = (int64_t)P.stages.size();
      comp_apply(true);
      stage_final(true);
      if (P.want_grad) stage_gradient();
      P.main_end = (int64_t)P.stages.size();
      const double sweep_flops = P.stats.exec_flops;
      const PlanStats counts = P.stats;
      comp_frozen_apply();
      if (scf) scf_segments();
      P.stats = counts;
      P.stats.exec_flops = sweep_flops;
    } else {
      stage_represent();
      stage_meanfield();
      if (cdvr) {  // CDVR::Update inside build, CDVR::apply added to Apply
        P.cdvr = true;
        P.stats.exec_flops += cdvr_plan(P, *cdvr, 0);
        stage_flops_mark = P.stats.exec_flops;
      }
      stage_apply();
      if (cdvr) {
        P.stats.exec_flops += cdvr_plan(P, *cdvr, 1);
        stage_flops_mark = P.stats.exec_flops;
      }
      if (P.want_grad) stage_environment();
      stage_final();
      if (P.want_grad) stage_gradient();
      P.main_end = (int64_t)P.stages.size();
    }
    P.mats_size = mats_cursor;
    P.keep_size = keep_cursor;
    count_reference_flops();
    P.stats.launches = P.main_end;
  }

 private:
  Plan& P;
  std::vector<NodeGeo>& nd;
  const OpTable& ops;
  const SopDesc& sop;
  bool grouped, compressed;
  bool scf = false;
  const CdvrDesc* cdvr = nullptr;
  int64_t budget;
  int n = 0, L = 0;
  std::vector<int> tops;  // roots of the forest, ascending
  bool is_top(int a) const { return nd[a].parent < 0; }
  // sparse activity: the terms active at each node (ascending) with their
  // represent / mean-field slots, and the active nodes of each term
  std::vector<std::vector<int>> node_terms;
  std::vector<std::vector<int64_t>> node_hslot, node_cslot;
  std::vector<std::vector<int>> term_nodes;
  std::vector<int> tin, tout;          // DFS interval of every node
  std::map<int, int> leaf_node;        // mode -> bottom node
  int idx_of(int l, int a) const {
    const auto& v = node_terms[a];
    auto it = std::lower_bound(v.begin(), v.end(), l);
    return (it != v.end() && *it == l) ? (int)(it - v.begin()) : -1;
  }
  bool act(int l, int a) const { return idx_of(l, a) >= 0; }
  int64_t hslot(int l, int a) const { return node_hslot[a][idx_of(l, a)]; }
  int64_t cslot(int l, int a) const { return node_cslot[a][idx_of(l, a)]; }
  bool inside_mode(int a, int m) const {
    const int leaf = leaf_node.at(m);
    return tin[a] <= tin[leaf] && tin[leaf] < tout[a];
  }
  std::vector<std::vector<int>> gkey;  // apply group of (term) per node, filled per node
  int64_t mats_cursor = 0;
  double stage_flops_mark = 0;
  int64_t stage_oz_ = 0;  // bytes of operand images assigned in the stage being emitted
  std::map<std::vector<int>, int64_t> hslot_of_key, cslot_of_key;

  double stage_bytes(int kind, int64_t t0, int64_t t1) const {
    double b = 0;
    for (int64_t t = t0; t < t1; ++t) {
      if (kind == ST_MP) {
        const auto& m = P.mp[t];
        double n_in = (double)m.before * m.a_in * m.after, n_out = (double)m.before * m.a_out * m.after;
        b += 16.0 * (n_in + n_out + (m.diag ? m.a_in : (double)m.a_in * m.a_out));
      } else if (kind == ST_HP) {
        const auto& h = P.hp[t];
        b += 16.0 * (2.0 * h.before * h.a * h.after + (double)h.a * h.a);
      } else if (kind == ST_ACC) {
        const auto& a = P.acc[t];
        double n = (double)a.rows * a.d;
        b += 16.0 * (n * (a.count + (a.add ? 2 : 1)) + (double)a.count * a.d * a.d);
      } else if (kind == ST_LIN) {
        const auto& l = P.lin[t];
        b += 16.0 * (double)l.d * l.d * (l.count + 1);
      } else if (kind == ST_EIG) {
        b += 16.0 * 2 * (double)P.eig[t].d * P.eig[t].d;
      } else if (kind == ST_PROJ) {
        b += 16.0 * 6 * (double)P.proj[t].d * P.proj[t].d;
      } else if (kind == ST_CVT) {
        b += 32.0 * (double)P.cvt[t].n;
      } else if (kind == ST_MM) {
        b += 16.0 * (double)P.mm[t].d * P.mm[t].d * (2 * P.mm[t].count + 1);
      }
    }
    return b;
  }

  Ref psi(int node) const { return Ref{B_PSI, nd[node].aoff}; }
  Ref hphi(int node) const { return Ref{B_HPHI, nd[node].aoff}; }
  Ref dpsi(int node) const { return Ref{B_DPSI, nd[node].aoff}; }
  Ref mat(int64_t off) const { return Ref{B_MATS, off}; }
  Ref opref(int op) const { return Ref{B_OPS, ops.off[op]}; }

  int64_t alloc_mat(int d) {
    int64_t o = mats_cursor;
    mats_cursor += align_up((int64_t)d * d);
    return o;
  }

  void geometry() {
    n = (int)nd.size();
    L = sop.n_terms;
    if (n == 0 || !nd[n - 1].top()) throw std::runtime_error("the last node must be a top node");
    int64_t off = 0, aoff = 0;
    for (int i = 0; i < n; ++i) {
      NodeGeo& g = nd[i];
      g.N = 1;
      for (int d : g.shape) g.N *= d;
      // node tensors stay packed in the arena (QuTree's TensorTree layout):
      // every kernel load is a naturally aligned 16-byte complex
      g.off = off;
      g.aoff = aoff;
      off += g.N;
      aoff += g.N;
      g.children.clear();
      if (g.shape.empty() || g.shape.back() < 1) throw std::runtime_error("empty node shape");
      if (g.shape.back() > 112) throw std::runtime_error("bond dimension above 112 is not supported");
      for (int d : g.shape)
        if (d < 1) throw std::runtime_error("non-positive dimension");
      if (g.N > (int64_t)1 << 30) throw std::runtime_error("node tensor too large");
    }
    P.psi_packed = off;
    P.psi_arena = aoff;
    for (int i = 0; i < n; ++i) {
      if (nd[i].parent >= 0) {
        if (nd[i].parent <= i) throw std::runtime_error("parents must follow their children");
        auto& ch = nd[nd[i].parent].children;
        if ((int)ch.size() <= nd[i].child_idx) ch.resize(nd[i].child_idx + 1, -1);
        ch[nd[i].child_idx] = i;
      } else {
        tops.push_back(i);  // a forest: every root closes one tree
      }
    }
    for (int i = 0; i < n; ++i) {
      NodeGeo& g = nd[i];
      if (g.bottom()) {
        if (g.shape.size() != 2) throw std::runtime_error("bottom nodes must have order 2");
        g.height = 0;
      } else {
        if ((int)g.children.size() + 1 != (int)g.shape.size())
          throw std::runtime_error("upper node order must be children + 1");
        int h = 0;
        for (size_t k = 0; k < g.children.size(); ++k) {
          int c = g.children[k];
          if (c < 0) throw std::runtime_error("missing child");
          if (nd[c].dup() != g.shape[k]) throw std::runtime_error("child bond mismatch");
          h = std::max(h, nd[c].height + 1);
        }
        g.height = h;
      }
    }
    for (int i = n - 1; i >= 0; --i) nd[i].depth = nd[i].top() ? 0 : nd[nd[i].parent].depth + 1;
  }

  void activity() {
    for (int i = 0; i < n; ++i)
      if (nd[i].bottom()) {
        if (leaf_node.count(nd[i].leaf_mode)) throw std::runtime_error("duplicate leaf mode");
        leaf_node[nd[i].leaf_mode] = i;
      }
    // DFS intervals: node a's subtree holds exactly the nodes with tin in [tin[a], tout[a])
    tin.assign(n, 0);
    tout.assign(n, 0);
    int clock = 0;
    std::vector<std::pair<int, int>> stack;
    for (int t : tops) {
      stack.push_back({t, 0});
      while (!stack.empty()) {
        auto& top_ = stack.back();
        const int a = top_.first;
        if (top_.second == 0) tin[a] = clock++;
        if (top_.second < (int)nd[a].children.size()) {
          const int c = nd[a].children[top_.second++];
          stack.push_back({c, 0});
        } else {
          tout[a] = clock;
          stack.pop_back();
        }
      }
    }
    node_terms.assign(n, {});
    term_nodes.assign(L, {});
    std::vector<int> stamp(n, -1);
    for (int l = 0; l < L; ++l) {
      if (sop.ptr[l + 1] <= sop.ptr[l]) throw std::runtime_error("empty SOP term");
      std::vector<int> nodes_l;
      for (int f = sop.ptr[l]; f < sop.ptr[l + 1]; ++f) {
        auto it = leaf_node.find(sop.mode[f]);
        if (it == leaf_node.end()) throw std::runtime_error("SOP factor on unknown mode");
        int op = sop.op[f];
        if (op < 0 || op >= (int)ops.kind.size()) throw std::runtime_error("bad operator id");
        if (ops.dim[op] != nd[it->second].shape[0])
          throw std::runtime_error("operator dim != leaf dim");
        for (int a = it->second; a >= 0 && stamp[a] != l; a = nd[a].parent) {
          stamp[a] = l;
          nodes_l.push_back(a);
        }
      }
      std::sort(nodes_l.begin(), nodes_l.end());
      int roots = 0;
      for (int a : nodes_l) {
        roots += is_top(a) ? 1 : 0;
        node_terms[a].push_back(l);
      }
      if (roots != 1) throw std::runtime_error("an SOP term acts on leaves of several trees");
      term_nodes[l] = std::move(nodes_l);
    }
  }

  // restriction of term l to the modes inside (in=true) or outside node a
  std::vector<int> key(int l, int a, bool in) const {
    std::vector<std::pair<int, int>> f;
    for (int x = sop.ptr[l]; x < sop.ptr[l + 1]; ++x) {
      int m = sop.mode[x];
      if (inside_mode(a, m) == in) f.push_back({m, sop.op[x]});
    }
    std::stable_sort(f.begin(), f.end(),
                     [](const std::pair<int, int>& u, const std::pair<int, int>& v) {
                       return u.first < v.first;
                     });
    std::vector<int> k;
    k.push_back(a);
    k.push_back(in ? 1 : 0);
    for (auto& p : f) k.push_back(p.first), k.push_back(p.second);
    return k;
  }

  void layout() {
    mats_cursor = 0;
    P.rho_off.assign(n, 0);
    P.rhoinv_off.assign(n, 0);
    P.u_off.assign(n, 0);
    P.s_off.assign(n, -1);
    P.sinv_off.assign(n, -1);
    P.d_off.assign(n, -1);
    P.p_off.assign(n, -1);
    P.m2_off.assign(n, -1);
    for (int i = 0; i < n; ++i) {
      int d = nd[i].dup();
      P.rho_off[i] = alloc_mat(d);
      P.rhoinv_off[i] = alloc_mat(d);
      P.u_off[i] = alloc_mat(d);
      P.max_eig_d = std::max(P.max_eig_d, d);
      if (!is_top(i)) {
        P.s_off[i] = alloc_mat(d);
        P.sinv_off[i] = alloc_mat(d);
        P.d_off[i] = alloc_mat(d);
        P.p_off[i] = alloc_mat(d);
        P.m2_off[i] = alloc_mat(d);
      }
    }
    P.rho64_off = P.rho_off;
    P.rhoinv64_off = P.rhoinv_off;
    P.s64_off = P.s_off;
    P.d64_off = P.d_off;
    P.m2_64_off = P.m2_off;
    if (P.prec >= 1) {
      for (int i = 0; i < n; ++i) {
        int d = nd[i].dup();
        P.rho64_off[i] = alloc_mat(d);
        P.rhoinv64_off[i] = alloc_mat(d);
      }
    }
    std::vector<int64_t> ident(n, -1);
    for (int t : tops) {
      int dt = nd[t].dup();
      P.tops.push_back(t);
      P.energy_dev_off.push_back(alloc_mat(dt));
      P.stop_dev_off.push_back(alloc_mat(dt));
      P.energy_off.push_back(P.prec >= 1 ? alloc_mat(dt) : P.energy_dev_off.back());
      P.stop_off.push_back(P.prec >= 1 ? alloc_mat(dt) : P.stop_dev_off.back());
      ident[t] = alloc_mat(dt);
      P.identities.push_back({ident[t], dt});
      P.identities.push_back({P.rho_off[t], dt});
    }
    P.term_nodes = term_nodes;
    if (compressed) {  // no per-term matrices
      P.per_term_mats = false;
      P.term_hslot.assign(L, {});
      P.term_cslot.assign(L, {});
      for (int l = 0; l < L; ++l) {
        P.term_hslot[l].assign(term_nodes[l].size(), -1);
        P.term_cslot[l].assign(term_nodes[l].size(), -1);
      }
      return;
    }
    // represent / mean-field slots
    node_hslot.assign(n, {});
    node_cslot.assign(n, {});
    for (int a = 0; a < n; ++a) {
      node_hslot[a].assign(node_terms[a].size(), -1);
      node_cslot[a].assign(node_terms[a].size(), -1);
      hslot_of_key.clear();  // keys carry the node, so slots never cross nodes
      cslot_of_key.clear();
      for (size_t i = 0; i < node_terms[a].size(); ++i) {
        const int l = node_terms[a][i];
        if (is_top(a)) {
          node_hslot[a][i] = -2;  // the reference leaves the top's represent matrix at zero
          node_cslot[a][i] = ident[a];
          continue;
        }
        std::vector<int> kin = grouped ? key(l, a, true) : std::vector<int>{a, 1, l};
        auto it = hslot_of_key.find(kin);
        if (it == hslot_of_key.end()) {
          int64_t o = alloc_mat(nd[a].dup());
          hslot_of_key[kin] = o;
          node_hslot[a][i] = o;
        } else {
          node_hslot[a][i] = it->second;
        }
        std::vector<int> kout = grouped ? key(l, a, false) : std::vector<int>{a, 0, l};
        auto jt = cslot_of_key.find(kout);
        if (jt == cslot_of_key.end()) {
          int64_t o = alloc_mat(nd[a].dup());
          cslot_of_key[kout] = o;
          node_cslot[a][i] = o;
        } else {
          node_cslot[a][i] = jt->second;
        }
      }
    }
    // per-term view for downloads (active nodes ascending)
    P.term_nodes = term_nodes;
    P.term_hslot.assign(L, {});
    P.term_cslot.assign(L, {});
    for (int l = 0; l < L; ++l)
      for (int a : term_nodes[l]) {
        P.term_hslot[l].push_back(hslot(l, a));
        P.term_cslot[l].push_back(cslot(l, a));
      }
  }

  // ---- stage emission ------------------------------------------------------
  // Blocks of the hole products [t0, t1): output tiles of up to 64 x 64 times
  // ranges of kchunk reduction rows, kchunk chosen so that the stage fills
  // about six blocks per SM, and at least 64 rows (below that, writing and
  // summing a partial tile costs more than its products); tasks with several
  // ranges get workspace slots for their partial tiles.  Returns whether any
  // task was split.
  bool hp_split(int64_t t0, int64_t t1, int64_t& tile0, int64_t& tile1) {
    constexpr int kTile = 64, kRows = 16;
    auto ntiles = [](const Plan::SHP& h) {
      return (int64_t)((h.a + kTile - 1) / kTile) * ((h.a + kTile - 1) / kTile);
    };
    // double-float plans with tensor-core hole products: the qualifying tasks
    // take the tensor-core path (hp_tensor_items), the others the tiles below
    std::vector<char> tc(t1 - t0, 0);
    if (P.hp_tensor)
      for (int64_t t = t0; t < t1; ++t)
        tc[t - t0] = hp_tc_eligible(P.hp[t].before, P.hp[t].a, P.hp[t].after, P.tune.hp);
    double work = 0;
    for (int64_t t = t0; t < t1; ++t)
      if (!tc[t - t0]) work += (double)ntiles(P.hp[t]) * P.hp[t].before * P.hp[t].after;
    const double target = 6.0 * 152;
    int64_t kc = (int64_t)std::ceil(work / target / kRows) * kRows;
    kc = std::max<int64_t>(kc, 64);
    tile0 = (int64_t)P.hp_tiles.size();
    int64_t ws = 0;
    bool split = false;
    for (int64_t t = t0; t < t1; ++t) {
      if (tc[t - t0]) continue;
      Plan::SHP& h = P.hp[t];
      // outputs per thread: the fewest (rows x cols) whose thread grid
      // ceil(m/rows) x ceil(m/cols) fits 256 threads and 64 staged columns
      hp_shape(std::min(h.a, kTile), &h.rows, &h.cols);
      const int64_t K = (int64_t)h.before * h.after;
      h.splits = (int)((K + kc - 1) / kc);
      h.kchunk = (int)std::min<int64_t>(K, kc);
      h.ws = 0;
      if (h.splits > 1) {
        h.ws = ws;
        ws += (int64_t)h.splits * h.a * h.a;
        split = true;
      }
    }
    if (P.hp_tensor && hp_tensor_items(t0, t1, tc, ws)) split = true;
    // tiles grouped by micro-tile shape: one launch per shape
    for (int shape = 0; shape < 16; ++shape) {
      const int64_t first = (int64_t)P.hp_tiles.size();
      for (int64_t t = t0; t < t1; ++t) {
        const Plan::SHP& h = P.hp[t];
        if (tc[t - t0] || (h.rows - 1) * 4 + (h.cols - 1) != shape) continue;
        for (int64_t y = 0; y < ntiles(h); ++y)
          for (int z = 0; z < h.splits; ++z) P.hp_tiles.push_back(make_int4((int)t, (int)y, z, 0));
      }
      const int64_t n = (int64_t)P.hp_tiles.size() - first;
      if (n > 0) P.hp_segs.push_back(make_int4(shape / 4 + 1, shape % 4 + 1, (int)first, (int)n));
    }
    tile1 = (int64_t)P.hp_tiles.size();
    P.hpw_size = std::max(P.hpw_size, ws);
    return split;
  }

  // Tensor-core hole products of the stage: the qualifying tasks (tc) in
  // groups of up to 128 / a tasks sharing A, one image of A per distinct A in
  // the stage's part of B_OZ, and one work item per chunk of the reduction.
  // A task of several chunks gets workspace slots for its partial tiles.
  // Returns whether any task was cut.
  bool hp_tensor_items(int64_t t0, int64_t t1, const std::vector<char>& tc, int64_t& ws) {
    const int64_t g0 = (int64_t)P.hp_tc_groups.size();
    std::map<std::tuple<int, int64_t, int, int, int>, int64_t> open, img;
    for (int64_t t = t0; t < t1; ++t) {
      if (!tc[t - t0]) continue;
      const Plan::SHP& h = P.hp[t];
      const auto key = std::make_tuple(h.A.buf, h.A.off, h.before, h.a, h.after);
      auto it = open.find(key);
      if (it == open.end() || P.hp_tc_groups[it->second].n >= std::min(kHpTcMembers, 128 / h.a)) {
        Plan::SHpTcGroup g;
        g.A = h.A;
        g.before = h.before;
        g.a = h.a;
        g.after = h.after;
        const int ap = (h.a + 7) & ~7, kc = hp_tc_kc(ap);
        g.nchunks = (int)(((int64_t)h.before * h.after + kc - 1) / kc);
        const int64_t gi = (int64_t)P.hp_tc_groups.size();
        auto im = img.find(key);
        if (im == img.end()) {  // this group's pre-pass writes A's images
          g.img = stage_oz_;
          stage_oz_ += g.nchunks * hp_tc_chunk_bytes(ap, kc / 16);
          img[key] = g.img;
          for (int c = 0; c < g.nchunks; ++c) P.hp_tc_imgs.push_back(make_int2((int)gi, c));
        } else {
          g.img = im->second;
        }
        g.ex = stage_oz_;  // the row exponents of this group's B, written by the items' pre-pass
        stage_oz_ += (int64_t)g.nchunks * 128;
        P.hp_tc_groups.push_back(g);
        open[key] = gi;
        it = open.find(key);
      }
      Plan::SHpTcGroup& g = P.hp_tc_groups[it->second];
      g.member[g.n++] = (int)t;
    }
    const int64_t g1 = (int64_t)P.hp_tc_groups.size();
    // one chunk per item: every unit stores its partial tiles (an item of
    // several chunks would add each chunk into them, whose loads of rows of
    // S stall the epilogue longer than the partial-tile sum takes)
    bool split = false;
    for (int64_t g = g0; g < g1; ++g) {
      const Plan::SHpTcGroup& G = P.hp_tc_groups[g];
      const int kc = hp_tc_kc((G.a + 7) & ~7);
      const int cpi = 1;
      const int splits = (G.nchunks + cpi - 1) / cpi;
      for (int m = 0; m < G.n; ++m) {
        Plan::SHP& h = P.hp[G.member[m]];
        h.splits = splits;
        h.kchunk = cpi * kc;
        h.ws = 0;
        if (splits > 1) {
          h.ws = ws;
          ws += (int64_t)splits * h.a * h.a;
          split = true;
        }
      }
      for (int z = 0; z < splits; ++z)
        P.hp_tc_items.push_back(make_int4((int)g, z, z * cpi, std::min(G.nchunks, (z + 1) * cpi)));
    }
    return split;
  }

  // Tensor-core accumulations of a stage [t0, t1): the qualifying tasks get
  // one item per block of 128 rows (the task's terms in order, one unit
  // each) and an image slot per term in the stage's part of B_OZ; their
  // classic tiles are dropped from [tile0, tile1).  Returns the new end of
  // the classic tiles; units = the units of all items.
  int64_t acc_tensor_items(int64_t t0, int64_t t1, int64_t tile0, int64_t tile1, int64_t& units) {
    std::vector<char> tc(t1 - t0, 0);
    units = 0;
    for (int64_t t = t0; t < t1; ++t) {
      Plan::SAcc& a = P.acc[t];
      if (a.count < 1 || !acc_tc_eligible(a.rows, a.d, P.tune.acc)) continue;
      tc[t - t0] = 1;
      a.tc_img = stage_oz_;
      stage_oz_ += (int64_t)a.count * hp_tc_chunk_bytes((a.d + 7) & ~7, 4);
      for (int s = 0; s < a.count; ++s) P.acc_tc_imgs.push_back(make_int2((int)t, s));
      for (int64_t b = 0; b * 128 < a.rows; ++b) {
        P.acc_tc_items.push_back(make_int4((int)t, (int)b, (int)units, 0));
        units += a.count;
      }
    }
    int64_t w = tile0;
    for (int64_t i = tile0; i < tile1; ++i) {
      const int4 tl = P.acc_tiles[i];
      if (tl.x >= t0 && tl.x < t1 && tc[tl.x - t0]) continue;
      P.acc_tiles[w++] = tl;
    }
    return w;
  }

  void emit_stage(int kind, int64_t t0, int64_t t1, int64_t tile0, int64_t tile1,
                  const char* name) {
    if (t1 <= t0) return;
    bool split = false;
    const int64_t seg0 = (int64_t)P.hp_segs.size();
    const int64_t hti0 = (int64_t)P.hp_tc_items.size(), htu0 = (int64_t)P.hp_tc_imgs.size();
    stage_oz_ = 0;  // operand images are rewritten by every stage's pre-pass
    if (kind == ST_HP) split = hp_split(t0, t1, tile0, tile1);
    const int64_t oz0 = (int64_t)P.mp_oz_tiles.size();
    const int64_t ozt0 = (int64_t)P.mp_oz_tasks.size();
    if (kind == ST_MP && P.mp_tensor) tile1 = mp_tensor_tiles(t0, t1, tile0, tile1);
    const int64_t ati0 = (int64_t)P.acc_tc_items.size(), atu0 = (int64_t)P.acc_tc_imgs.size();
    int64_t atc_units = 0;
    if (kind == ST_ACC && P.hp_tensor) tile1 = acc_tensor_items(t0, t1, tile0, tile1, atc_units);
    P.oz_bytes = std::max(P.oz_bytes, stage_oz_);
    const double f1 = P.stats.exec_flops;
    Stage s;
    s.flops = f1 - stage_flops_mark;
    s.bytes = stage_bytes(kind, t0, t1);
    stage_flops_mark = f1;
    s.kind = kind;
    s.first_task = t0;
    s.n_tasks = t1 - t0;
    s.first_tile = tile0;
    s.n_tiles = tile1 - tile0;
    s.name = name;
    s.aux = split ? 1 : 0;
    s.seg0 = (int)seg0;
    s.nseg = (int)((int64_t)P.hp_segs.size() - seg0);
    s.oz0 = oz0;
    s.noz = (int64_t)P.mp_oz_tiles.size() - oz0;
    s.ozt0 = ozt0;
    s.nozt = (int64_t)P.mp_oz_tasks.size() - ozt0;
    s.hti0 = hti0;
    s.nhti = (int64_t)P.hp_tc_items.size() - hti0;
    s.htu0 = htu0;
    s.nhtu = (int64_t)P.hp_tc_imgs.size() - htu0;
    s.ati0 = ati0;
    s.nati = (int64_t)P.acc_tc_items.size() - ati0;
    s.atu0 = atu0;
    s.natu = (int64_t)P.acc_tc_imgs.size() - atu0;
    s.atc_units = atc_units;
    P.stages.push_back(s);
  }

  // Tensor-core mode products: the qualifying tasks of a stage [t0, t1) get
  // tiles of kMpOzSub x kMpOzRows rows; their classic tiles are dropped from
  // [tile0, tile1).  Returns the new end of the classic tiles.
  int64_t mp_tensor_tiles(int64_t t0, int64_t t1, int64_t tile0, int64_t tile1) {
    std::vector<char> oz(t1 - t0, 0);
    for (int64_t t = t0; t < t1; ++t) {
      auto& m = P.mp[t];
      if (m.diag || !mp_tc_eligible(m.a_in, m.a_out, P.tune.mp)) continue;
      oz[t - t0] = 1;
      m.oz_h = stage_oz_;
      // double-float plans: the sum-of-products kernel's image of alpha h;
      // complex64 plans: the split-TF32 image
      stage_oz_ += P.hp_tensor ? hp_tc_chunk_bytes((m.a_out + 7) & ~7, 4) : mp_oz_h_bytes();
      P.mp_oz_tasks.push_back((int)t);
      const int64_t rows = (int64_t)m.before * m.after;
      for (int64_t r = 0; r * kMpOzRows * kMpOzSub < rows; ++r)
        P.mp_oz_tiles.push_back(make_int2((int)t, (int)r));
    }
    int64_t w = tile0;
    for (int64_t i = tile0; i < tile1; ++i) {
      const int2 tl = P.mp_tiles[i];
      if (tl.x >= t0 && tl.x < t1 && oz[tl.x - t0]) continue;
      P.mp_tiles[w++] = tl;
    }
    return w;
  }

  void add_mp(Ref in, Ref out, Ref h, double2 alpha, int node, int mode, bool diag) {
    const NodeGeo& g = nd[node];
    Plan::SMP t;
    t.in = in;
    t.out = out;
    t.h = h;
    t.alpha = alpha;
    t.before = (int)g.before(mode);
    t.a_in = g.shape[mode];
    t.a_out = g.shape[mode];
    t.after = (int)g.after(mode);
    t.diag = diag ? 1 : 0;
    int task = (int)P.mp.size();
    P.mp.push_back(t);
    const int64_t slots = (int64_t)t.before * ((t.a_out + 3) / 4) * t.after;
    for (int64_t s = 0; s < slots; s += kMpTile) P.mp_tiles.push_back(make_int2(task, (int)s));
    P.stats.exec_flops += diag ? 6.0 * g.N : 8.0 * g.N * g.shape[mode];
  }

  void add_cvt(Ref src, Ref dst, int64_t n, int dir) {
    Plan::SCvt t;
    t.src = src;
    t.dst = dst;
    t.n = n;
    t.dir = dir;
    int task = (int)P.cvt.size();
    P.cvt.push_back(t);
    for (int64_t s = 0; s < n; s += 2048) P.cvt_tiles.push_back(make_int2(task, (int)s));
  }

  // one conversion stage over several matrices
  void cvt_mats(const std::vector<int64_t>& src, const std::vector<int64_t>& dst, int dir,
                const char* name, bool skip_top) {
    int64_t c0 = (int64_t)P.cvt.size(), t0 = (int64_t)P.cvt_tiles.size();
    for (int a = 0; a < n; ++a) {
      if (skip_top && is_top(a)) continue;
      if (src[a] < 0 || dst[a] < 0) continue;
      add_cvt(mat(src[a]), mat(dst[a]), (int64_t)nd[a].dup() * nd[a].dup(), dir);
    }
    emit_stage(ST_CVT, c0, (int64_t)P.cvt.size(), t0, (int64_t)P.cvt_tiles.size(), name);
  }

  void add_hp(Ref A, Ref B, Ref S, int node, int mode) {
    const NodeGeo& g = nd[node];
    Plan::SHP t;
    t.A = A;
    t.B = B;
    t.S = S;
    t.before = (int)g.before(mode);
    t.a = g.shape[mode];
    t.after = (int)g.after(mode);
    P.hp.push_back(t);  // tiles are cut per stage (hp_split)
    P.stats.exec_flops += 8.0 * g.N * g.shape[mode];
  }

  void add_acc(Ref out, bool alpha_param, double2 alpha, int node,
               const std::vector<Plan::SAccTerm>& terms, bool add) {
    const NodeGeo& g = nd[node];
    Plan::SAcc t;
    t.out = out;
    t.alpha_param = alpha_param;
    t.alpha = alpha;
    t.d = g.dup();
    t.rows = (int)(g.N / t.d);
    t.first = (int)P.acc_terms.size();
    t.count = (int)terms.size();
    t.add = add ? 1 : 0;
    for (auto& x : terms) P.acc_terms.push_back(x);
    int task = (int)P.acc.size();
    P.acc.push_back(t);
    for (int r0 = 0; r0 < t.rows; r0 += kAccRows)
      for (int j0 = 0; j0 < t.d; j0 += kAccCols) P.acc_tiles.push_back(make_int4(task, r0, j0, 0));
    for (auto& x : terms) P.stats.exec_flops += (x.H.buf < 0 ? 2.0 : 8.0 * t.d) * g.N;
  }

  // out = sum_t A_t op(B_t), d x d (op = transpose when trans_b)
  void add_mm(Ref out, int d, const std::vector<Plan::SMMTerm>& terms, bool trans_b) {
    Plan::SMM t;
    t.out = out;
    t.d = d;
    t.first = (int)P.mm_terms.size();
    t.count = (int)terms.size();
    t.trans_b = trans_b ? 1 : 0;
    for (auto& x : terms) P.mm_terms.push_back(x);
    const int task = (int)P.mm.size();
    P.mm.push_back(t);
    for (int e0 = 0; e0 < d * d; e0 += 256) P.mm_tiles.push_back(make_int2(task, e0));
    P.stats.exec_flops += 8.0 * d * d * d * (double)terms.size();
  }

  // Run a list of chains as one group (split into chunks by the scratch budget).
  void run_items(std::vector<Item>& items, const char* name, std::vector<char>* acc_started) {
    size_t i = 0;
    while (i < items.size()) {
      // chunk [i, j)
      int64_t cursor = 0;
      size_t j = i;
      std::vector<std::pair<int64_t, int64_t>> bufs;  // per item buf0, buf1 offsets
      while (j < items.size()) {
        const Item& it = items[j];
        int64_t need = 0;
        int nb = (int)std::min<size_t>(2, it.ops.size());
        need = nb * align_up(nd[it.node].N);
        if (j > i && cursor + need > budget) break;
        bufs.push_back({nb > 0 ? cursor : -1, nb > 1 ? cursor + align_up(nd[it.node].N) : -1});
        cursor += need;
        ++j;
      }
      P.scratch_size = std::max(P.scratch_size, cursor);
      size_t maxops = 0;
      for (size_t k = i; k < j; ++k) maxops = std::max(maxops, items[k].ops.size());
      for (size_t pos = 0; pos < maxops; ++pos) {
        int64_t t0 = (int64_t)P.mp.size(), tile0 = (int64_t)P.mp_tiles.size();
        for (size_t k = i; k < j; ++k) {
          const Item& it = items[k];
          if (pos >= it.ops.size()) continue;
          const auto& b = bufs[k - i];
          Ref in = pos == 0 ? it.in : Ref{B_SCR, (pos - 1) % 2 == 0 ? b.first : b.second};
          Ref out{B_SCR, pos % 2 == 0 ? b.first : b.second};
          const COp& op = it.ops[pos];
          add_mp(in, out, op.mat, op.alpha, it.node, op.mode, op.kind == 1);
        }
        emit_stage(ST_MP, t0, (int64_t)P.mp.size(), tile0, (int64_t)P.mp_tiles.size(), name);
      }
      // finals: hole products
      {
        int64_t t0 = (int64_t)P.hp.size(), tile0 = (int64_t)P.hp_tiles.size();
        for (size_t k = i; k < j; ++k) {
          const Item& it = items[k];
          if (it.fin != 0) continue;
          const auto& b = bufs[k - i];
          size_t no = it.ops.size();
          Ref x = no == 0 ? it.in : Ref{B_SCR, (no - 1) % 2 == 0 ? b.first : b.second};
          add_hp(psi(it.node), x, it.S, it.node, it.hp_mode);
        }
        emit_stage(ST_HP, t0, (int64_t)P.hp.size(), tile0, (int64_t)P.hp_tiles.size(), name);
      }
      // finals: accumulation per node
      {
        int64_t t0 = (int64_t)P.acc.size(), tile0 = (int64_t)P.acc_tiles.size();
        std::map<int, std::vector<Plan::SAccTerm>> per_node;
        for (size_t k = i; k < j; ++k) {
          const Item& it = items[k];
          if (it.fin != 1) continue;
          const auto& b = bufs[k - i];
          size_t no = it.ops.size();
          Ref x = no == 0 ? it.in : Ref{B_SCR, (no - 1) % 2 == 0 ? b.first : b.second};
          per_node[it.acc_node].push_back(Plan::SAccTerm{it.accH, x});
        }
        for (auto& kv : per_node) {
          bool add = (*acc_started)[kv.first] != 0;
          add_acc(hphi(kv.first), false, c2(1.0, 0.0), kv.first, kv.second, add);
          (*acc_started)[kv.first] = 1;
        }
        emit_stage(ST_ACC, t0, (int64_t)P.acc.size(), tile0, (int64_t)P.acc_tiles.size(), name);
      }
      i = j;
    }
  }

  void stage_density() {
    int maxdepth = 0;
    for (auto& g : nd) maxdepth = std::max(maxdepth, g.depth);
    for (int d = 1; d <= maxdepth; ++d) {
      std::vector<Item> items;
      for (int a = 0; a < n; ++a) {
        if (nd[a].depth != d) continue;
        int p = nd[a].parent;
        Item it;
        it.node = p;
        it.in = psi(p);
        if (!nd[p].top())
          it.ops.push_back(COp{0, nd[p].last(), mat(P.rho_off[p]), c2(1, 0)});
        it.fin = 0;
        it.S = mat(P.rho_off[a]);
        it.hp_mode = nd[a].child_idx;
        items.push_back(it);
      }
      run_items(items, "density", nullptr);
    }
  }

  void stage_inverse() {
    if (P.prec >= 1) cvt_mats(P.rho_off, P.rho64_off, 1, "rho-to-f64", false);
    int64_t t0 = (int64_t)P.eig.size();
    for (int a = 0; a < n; ++a) {
      Plan::SEig e;
      e.rho = mat(P.rho64_off[a]);
      e.rhoinv = mat(P.rhoinv64_off[a]);
      e.U = mat(P.u_off[a]);
      e.d = nd[a].dup();
      P.eig.push_back(e);
    }
    emit_stage(ST_EIG, t0, (int64_t)P.eig.size(), t0, (int64_t)P.eig.size(), "inverse");
    if (P.prec >= 1) cvt_mats(P.rhoinv64_off, P.rhoinv_off, 0, "rhoinv-to-df", false);
  }

  // operators of term l at node a (represent / apply chain body)
  std::vector<COp> body(int l, int a, double2 alpha) const {
    std::vector<COp> o;
    const NodeGeo& g = nd[a];
    if (g.bottom()) {
      for (int f = sop.ptr[l]; f < sop.ptr[l + 1]; ++f) {
        if (sop.mode[f] != g.leaf_mode) continue;
        int op = sop.op[f];
        o.push_back(COp{ops.kind[op] == 0 ? 0 : 1, 0, opref(op), c2(1, 0)});
      }
    } else {
      for (size_t k = 0; k < g.children.size(); ++k) {
        int c = g.children[k];
        if (!act(l, c)) continue;
        o.push_back(COp{0, (int)k, mat(hslot(l, c)), c2(1, 0)});
      }
    }
    if (!o.empty()) o[0].alpha = alpha;
    return o;
  }

  void stage_represent() {
    int maxh = 0;
    for (int t : tops) maxh = std::max(maxh, nd[t].height);
    for (int h = 0; h < maxh; ++h) {
      std::vector<Item> items;
      std::set<int64_t> done;
      for (int a = 0; a < n; ++a) {
        if (nd[a].height != h || is_top(a)) continue;
        for (size_t i = 0; i < node_terms[a].size(); ++i) {
          const int l = node_terms[a][i];
          int64_t slot = node_hslot[a][i];
          if (!done.insert(slot).second) continue;
          Item it;
          it.node = a;
          it.in = psi(a);
          it.ops = body(l, a, c2(1, 0));
          it.fin = 0;
          it.S = mat(slot);
          it.hp_mode = nd[a].last();
          items.push_back(it);
        }
      }
      P.stats.rep_chains += (int64_t)items.size();
      run_items(items, "represent", nullptr);
    }
  }

  void stage_meanfield() {
    int maxdepth = 0;
    for (auto& g : nd) maxdepth = std::max(maxdepth, g.depth);
    for (int d = 1; d <= maxdepth; ++d) {
      std::vector<Item> items;
      std::set<int64_t> done;
      for (int a = 0; a < n; ++a) {
        if (nd[a].depth != d) continue;
        int p = nd[a].parent;
        for (size_t i = 0; i < node_terms[a].size(); ++i) {
          const int l = node_terms[a][i];
          int64_t slot = node_cslot[a][i];
          if (!done.insert(slot).second) continue;
          Item it;
          it.node = p;
          it.in = psi(p);
          const NodeGeo& gp = nd[p];
          for (size_t k = 0; k < gp.children.size(); ++k) {
            int c = gp.children[k];
            if ((int)k == nd[a].child_idx || !act(l, c)) continue;
            it.ops.push_back(COp{0, (int)k, mat(hslot(l, c)), c2(1, 0)});
          }
          if (!gp.top()) it.ops.push_back(COp{0, gp.last(), mat(cslot(l, p)), c2(1, 0)});
          it.fin = 0;
          it.S = mat(slot);
          it.hp_mode = nd[a].child_idx;
          items.push_back(it);
        }
      }
      P.stats.mf_chains += (int64_t)items.size();
      run_items(items, "meanfield", nullptr);
    }
  }

  void stage_apply() {
    P.apply_begin = (int64_t)P.stages.size();
    // group terms per node by their inside restriction; G_g = sum_l c_l H_l
    std::vector<Item> items;
    int64_t lin0 = (int64_t)P.lin.size();
    for (int a = 0; a < n; ++a) {
      std::map<std::vector<int>, std::vector<int>> groups;
      std::vector<std::vector<int>> order;
      for (int l : node_terms[a]) {
        std::vector<int> k = grouped ? key(l, a, true) : std::vector<int>{a, 1, l};
        auto it = groups.find(k);
        if (it == groups.end()) {
          groups[k] = {l};
          order.push_back(k);
        } else {
          it->second.push_back(l);
        }
      }
      int d = nd[a].dup();
      for (auto& k : order) {
        const auto& terms = groups[k];
        int64_t g = alloc_mat(d);
        Plan::SLin lt;
        lt.out = mat(g);
        lt.d = d;
        lt.first = (int)P.lin_terms.size();
        lt.count = (int)terms.size();
        for (int l : terms) P.lin_terms.push_back(Plan::SLinTerm{sop.coeff[l], mat(cslot(l, a))});
        P.lin.push_back(lt);
        Item it;
        it.node = a;
        it.in = psi(a);
        it.ops = body(terms[0], a, c2(1, 0));
        it.fin = 1;
        it.acc_node = a;
        it.accH = mat(g);
        items.push_back(it);
      }
    }
    emit_stage(ST_LIN, lin0, (int64_t)P.lin.size(), lin0, (int64_t)P.lin.size(), "apply-sum");
    P.stats.app_chains += (int64_t)items.size();
    std::vector<char> started(n, 0);
    run_items(items, "apply", &started);
    // nodes no SOP term reaches: H Phi = 0 there (Apply's empty sum)
    int64_t t0 = (int64_t)P.acc.size(), tile0 = (int64_t)P.acc_tiles.size();
    for (int a = 0; a < n; ++a)
      if (!started[a]) add_acc(hphi(a), false, c2(1.0, 0.0), a, {}, false);
    emit_stage(ST_ACC, t0, (int64_t)P.acc.size(), tile0, (int64_t)P.acc_tiles.size(), "apply-zero");
  }

  // fused (compressed sweep only): H Phi of non-top nodes is never formed.
  // With hphi(a) = Y(a) x_last rho_a + sum_u X(a,u) x_last C(a,u),
  //   D_a = Phi_a^dag hphi_a = Block(a) rho_a^T + sum_u H(a,u) C(a,u)^T
  // (a hole product on the last index commutes with last-index products), and
  //   hphi_a x_last rhoinv_a = Y x_last (rhoinv rho) + sum_u X_u x_last (rhoinv C_u),
  // so the derivative is one accumulation over the kept chain outputs.
  std::vector<std::vector<int64_t>> fused_g;  // per node: rhoinv rho, then rhoinv C(a,u)

  void stage_final(bool fused = false) {
    // overlaps S = Phi^dag Phi and D = Phi^dag (H Phi) of every node
    int64_t t0 = (int64_t)P.hp.size(), tile0 = (int64_t)P.hp_tiles.size();
    for (int a = 0; a < n; ++a) {
      if (is_top(a)) {
        const size_t k = std::find(tops.begin(), tops.end(), a) - tops.begin();
        add_hp(psi(a), hphi(a), mat(P.energy_dev_off[k]), a, nd[a].last());
        add_hp(psi(a), psi(a), mat(P.stop_dev_off[k]), a, nd[a].last());
      } else {
        add_hp(psi(a), psi(a), mat(P.s_off[a]), a, nd[a].last());
        if (!fused) add_hp(psi(a), hphi(a), mat(P.d_off[a]), a, nd[a].last());
      }
    }
    emit_stage(ST_HP, t0, (int64_t)P.hp.size(), tile0, (int64_t)P.hp_tiles.size(), "overlaps");
    if (fused) {
      fused_g.assign(n, {});
      const int64_t m0 = (int64_t)P.mm.size(), mt0 = (int64_t)P.mm_tiles.size();
      for (int a = 0; a < n; ++a) {
        if (is_top(a)) continue;
        const int d = nd[a].dup();
        std::vector<Plan::SMMTerm> dt;
        if (!internal[a].empty()) dt.push_back(Plan::SMMTerm{mat(block_slot[a]), mat(P.rho_off[a])});
        for (auto& b : bk[a]) dt.push_back(Plan::SMMTerm{mat(b.hslot), mat(b.cslot)});
        add_mm(mat(P.d_off[a]), d, dt, true);
        if (!internal[a].empty()) {
          fused_g[a].push_back(alloc_mat(d));
          add_mm(mat(fused_g[a].back()), d, {Plan::SMMTerm{mat(P.rhoinv_off[a]), mat(P.rho_off[a])}}, false);
        } else {
          fused_g[a].push_back(-1);
        }
        for (auto& b : bk[a]) {
          fused_g[a].push_back(alloc_mat(d));
          add_mm(mat(fused_g[a].back()), d, {Plan::SMMTerm{mat(P.rhoinv_off[a]), mat(b.cslot)}}, false);
        }
      }
      emit_stage(ST_MM, m0, (int64_t)P.mm.size(), mt0, (int64_t)P.mm_tiles.size(), "overlaps-fused");
    }
    if (P.prec >= 1) {  // the tree energies to complex128 (qt_energy reads them)
      int64_t c0 = (int64_t)P.cvt.size(), ct0 = (int64_t)P.cvt_tiles.size();
      for (size_t k = 0; k < tops.size(); ++k) {
        int dt = nd[tops[k]].dup();
        add_cvt(mat(P.energy_dev_off[k]), mat(P.energy_off[k]), (int64_t)dt * dt, 1);
        add_cvt(mat(P.stop_dev_off[k]), mat(P.stop_off[k]), (int64_t)dt * dt, 1);
      }
      emit_stage(ST_CVT, c0, (int64_t)P.cvt.size(), ct0, (int64_t)P.cvt_tiles.size(), "energies-to-f64");
    }

    int64_t p0 = (int64_t)P.proj.size();
    for (int a = 0; a < n; ++a) {
      if (is_top(a)) continue;
      Plan::SProj pj;
      // the projector runs in the plan's arithmetic on its own matrices
      pj.S = mat(P.s_off[a]);
      pj.D = mat(P.d_off[a]);
      pj.rhoinv = mat(P.rhoinv_off[a]);
      pj.Sinv = mat(P.sinv_off[a]);
      pj.P = mat(P.p_off[a]);
      pj.M2 = mat(P.m2_off[a]);
      pj.d = nd[a].dup();
      P.proj.push_back(pj);
      P.stats.exec_flops += 3 * 8.0 * pj.d * pj.d * pj.d;
    }
    emit_stage(ST_PROJ, p0, (int64_t)P.proj.size(), p0, (int64_t)P.proj.size(), "projector");

    // dPsi = -i*phase * (H Phi - Phi P) rhoinv^T  (non-top);  -i*phase * H Phi (top)
    int64_t a0 = (int64_t)P.acc.size(), atile0 = (int64_t)P.acc_tiles.size();
    for (int a = 0; a < n; ++a) {
      std::vector<Plan::SAccTerm> terms;
      if (is_top(a)) {
        terms.push_back(Plan::SAccTerm{Ref{-1, 0}, hphi(a)});
      } else if (fused) {
        if (fused_g[a][0] >= 0) terms.push_back(Plan::SAccTerm{mat(fused_g[a][0]), Yref[a]});
        for (size_t u = 0; u < bk[a].size(); ++u)
          terms.push_back(Plan::SAccTerm{mat(fused_g[a][u + 1]), bk[a][u].X});
        terms.push_back(Plan::SAccTerm{mat(P.m2_off[a]), psi(a)});
      } else {
        terms.push_back(Plan::SAccTerm{mat(P.rhoinv_off[a]), hphi(a)});
        terms.push_back(Plan::SAccTerm{mat(P.m2_off[a]), psi(a)});
      }
      add_acc(dpsi(a), true, c2(0, 0), a, terms, false);
    }
    emit_stage(ST_ACC, a0, (int64_t)P.acc.size(), atile0, (int64_t)P.acc_tiles.size(), "derivative");
    if (P.prec >= 1) {
      int64_t c0 = (int64_t)P.cvt.size(), ct0 = (int64_t)P.cvt_tiles.size();
      add_cvt(Ref{B_DPSI, 0}, Ref{B_DPSI64, 0}, P.psi_packed, 1);
      emit_stage(ST_CVT, c0, (int64_t)P.cvt.size(), ct0, (int64_t)P.cvt_tiles.size(), "dpsi-out");
    }
  }

  // ---- energy gradient (orthonormal gauge) --------------------------------
  // dE/dPhi_n^* = (Apply(n) + Phi_n x_last Eout[n] - E Phi_n x_last rho[n]) / S00
  // where Eout[n] is the mean field of every term acting entirely outside
  // node n -- the terms the reference's sparse sweep leaves out because the
  // MCTDH projector removes them.  Top-down: at the parent p, Eout[n] sums
  //   (a) p's own environment Eout[p] on the parent index, and
  //   (b) every term active at p but not at n: its represent matrices on the
  //       siblings of n and its mean field H_l[p] on the parent index.
  // Terms with the same sibling restriction share one chain; their mean
  // fields are summed first (and Eout[p] joins the all-identity group).
  std::vector<int64_t> eout_off;
  void stage_environment() {
    eout_off.assign(n, -1);
    int maxdepth = 0;
    for (auto& g : nd) maxdepth = std::max(maxdepth, g.depth);
    for (int dep = 1; dep <= maxdepth; ++dep) {
      std::vector<Item> items;
      int64_t lin0 = (int64_t)P.lin.size();
      std::vector<std::pair<int, std::vector<int64_t>>> sums;  // node -> temp slots
      for (int a = 0; a < n; ++a) {
        if (nd[a].depth != dep) continue;
        const int p = nd[a].parent;
        const NodeGeo& gp = nd[p];
        eout_off[a] = alloc_mat(nd[a].dup());
        // group the terms active at p but not at a by their sibling restrictions
        std::map<std::vector<int>, std::vector<int>> groups;
        std::vector<std::vector<int>> order;
        for (int l : node_terms[p]) {
          if (act(l, a)) continue;
          std::vector<int> k;
          for (size_t c = 0; c < gp.children.size(); ++c) {
            const int ch = gp.children[c];
            if (ch == a) continue;
            if (act(l, ch)) {
              std::vector<int> kk = key(l, ch, true);
              k.insert(k.end(), kk.begin(), kk.end());
            }
            k.push_back(-1);
          }
          auto it = groups.find(k);
          if (it == groups.end()) {
            groups[k] = {l};
            order.push_back(k);
          } else {
            it->second.push_back(l);
          }
        }
        std::vector<int> idkey;
        for (size_t c = 0; c + 1 < gp.children.size(); ++c) idkey.push_back(-1);
        if (!gp.top() && !groups.count(idkey)) {
          groups[idkey] = {};
          order.push_back(idkey);
        }
        std::vector<int64_t> temps;
        const int dp = gp.dup();
        for (auto& k : order) {
          const auto& terms = groups[k];
          // G = sum_l c_l H_l[p] (+ Eout[p] for the all-identity group)
          int64_t g = alloc_mat(dp);
          Plan::SLin lt;
          lt.out = mat(g);
          lt.d = dp;
          lt.first = (int)P.lin_terms.size();
          for (int l : terms) P.lin_terms.push_back(Plan::SLinTerm{sop.coeff[l], mat(cslot(l, p))});
          if (k == idkey && !gp.top()) P.lin_terms.push_back(Plan::SLinTerm{c2(1, 0), mat(eout_off[p])});
          lt.count = (int)P.lin_terms.size() - lt.first;
          P.lin.push_back(lt);
          Item it;
          it.node = p;
          it.in = psi(p);
          if (!terms.empty()) {
            const int l0 = terms[0];
            for (size_t c = 0; c < gp.children.size(); ++c) {
              const int ch = gp.children[c];
              if (ch == a || !act(l0, ch)) continue;
              it.ops.push_back(COp{0, (int)c, mat(hslot(l0, ch)), c2(1, 0)});
            }
          }
          it.ops.push_back(COp{0, gp.last(), mat(g), c2(1, 0)});
          it.fin = 0;
          int64_t tslot = alloc_mat(nd[a].dup());
          it.S = mat(tslot);
          it.hp_mode = nd[a].child_idx;
          items.push_back(it);
          temps.push_back(tslot);
        }
        sums.push_back({a, temps});
      }
      emit_stage(ST_LIN, lin0, (int64_t)P.lin.size(), lin0, (int64_t)P.lin.size(), "environment-sums");
      run_items(items, "environment", nullptr);
      int64_t s0 = (int64_t)P.lin.size();
      for (auto& pr : sums) {
        Plan::SLin lt;
        lt.out = mat(eout_off[pr.first]);
        lt.d = nd[pr.first].dup();
        lt.first = (int)P.lin_terms.size();
        for (int64_t t : pr.second) P.lin_terms.push_back(Plan::SLinTerm{c2(1, 0), mat(t)});
        lt.count = (int)pr.second.size();
        P.lin.push_back(lt);
      }
      emit_stage(ST_LIN, s0, (int64_t)P.lin.size(), s0, (int64_t)P.lin.size(), "environment");
    }
  }

  void stage_gradient() {
    int64_t g0 = (int64_t)P.grad.size();
    std::vector<int64_t> m3(n), alpha(tops.size());
    for (size_t k = 0; k < tops.size(); ++k) alpha[k] = alloc_mat(1);
    std::vector<int> tree_of(n, -1);
    for (size_t k = 0; k < tops.size(); ++k)
      for (int a = 0; a < n; ++a)
        if (tin[a] >= tin[tops[k]] && tin[a] < tout[tops[k]]) tree_of[a] = (int)k;
    for (int a = 0; a < n; ++a) {
      const int k = tree_of[a];
      Plan::SGrad t;
      m3[a] = alloc_mat(nd[a].dup());
      t.eout = is_top(a) ? Ref{-1, 0} : mat(eout_off[a]);
      t.rho = mat(P.rho_off[a]);
      t.m3 = mat(m3[a]);
      t.h00 = mat(P.energy_off[k]);
      t.s00 = mat(P.stop_off[k]);
      t.alpha = mat(alpha[k]);
      t.d = nd[a].dup();
      t.write_alpha = is_top(a) ? 1 : 0;
      P.grad.push_back(t);
    }
    emit_stage(ST_GRAD, g0, (int64_t)P.grad.size(), g0, (int64_t)P.grad.size(), "gradient-prep");
    int64_t a0 = (int64_t)P.acc.size(), atile0 = (int64_t)P.acc_tiles.size();
    for (int a = 0; a < n; ++a) {
      std::vector<Plan::SAccTerm> terms;
      if (compressed && !is_top(a)) {  // Apply(a) from the kept chains (H Phi is not formed)
        if (!internal[a].empty()) terms.push_back(Plan::SAccTerm{mat(P.rho_off[a]), Yref[a]});
        for (auto& b : bk[a]) terms.push_back(Plan::SAccTerm{mat(b.cslot), b.X});
      } else {
        terms.push_back(Plan::SAccTerm{Ref{-1, 0}, hphi(a)});
      }
      terms.push_back(Plan::SAccTerm{mat(m3[a]), psi(a)});
      add_acc(Ref{B_GRAD, nd[a].aoff}, true, c2(1, 0), a, terms, false);
      P.acc.back().alpha_ref = mat(alpha[tree_of[a]]);
    }
    emit_stage(ST_ACC, a0, (int64_t)P.acc.size(), atile0, (int64_t)P.acc_tiles.size(), "gradient");
    if (P.prec >= 1) {
      int64_t c0 = (int64_t)P.cvt.size(), ct0 = (int64_t)P.cvt_tiles.size();
      add_cvt(Ref{B_GRAD, 0}, Ref{B_GRAD64, 0}, P.psi_packed, 1);
      emit_stage(ST_CVT, c0, (int64_t)P.cvt.size(), ct0, (int64_t)P.cvt_tiles.size(), "gradient-out");
    }
  }

  // ---- compressed plan (QT_PLAN_COMPRESSED) ------------------------------
  // At every node a the active terms split into internal terms (no factor
  // outside a's subtree) and boundary terms.  Boundary terms with the same
  // inside restriction u share
  //   X(a,u) = (u's child represent matrices or leaf operators) Phi_a  [kept]
  //   H(a,u) = hole_last(Phi_a, X(a,u))                               [represent]
  //   C(a,u) = sum_l c_l MF_l(a)                          [their mean fields, summed]
  // and the internal terms share
  //   Y(a) = sum_l c_l body_l Phi_a  [kept],   Block(a) = hole_last(Phi_a, Y(a)).
  // The mean field of an internal term is the density matrix rho_a (both obey
  // the same top-down recursion from the identity at the top), so
  //   Apply(a) = Y(a) x_last rho_a + sum_u X(a,u) x_last C(a,u),   Apply(top) = Y(top).
  // Y(a) sums Block(c) on every child leg c and, for terms that span several
  // children, chains of cover groups: terms sharing all child factors but one
  // share one chain whose free factor is the summed sum_l c_l H_l on that leg.
  // C(a,u) is built at the parent p: terms internal to p contribute their
  // sibling represent matrices applied to Phi_p x_last rho_p (cover groups
  // over the sibling legs); terms reaching outside p contribute their sibling
  // matrices on Phi_p and C(p,w) on the parent index, w their restriction to p.
  // Every matrix is still a sum over the reference's per-term objects
  // (TreeFunctions::represent / contraction); only the order of the sums
  // changes.  Per-term matrices are not materialised.
  struct BKey {
    std::vector<int> terms;  // boundary terms with this inside restriction
    int64_t hslot = -1, cslot = -1;
    Ref X;
  };
  struct Chain {
    Ref in;
    std::vector<COp> ops;
    Ref H;  // factor on the last index applied when the chains are summed; buf -1: none
  };
  struct Job {
    int node = -1;  // geometry of every tensor of the job
    std::vector<Chain> chains;
    Ref out;  // destination of the summed chains; buf -1: scratch
    Ref S;    // buf >= 0: hole product of Phi_node with the sum over hp_mode into S
    int hp_mode = 0;
  };
  struct Group {
    int free_leg;
    std::vector<int> members;
  };
  std::vector<std::vector<BKey>> bk;
  std::vector<std::vector<int>> node_bk;  // aligned with node_terms: boundary key, -1 internal
  std::vector<std::vector<int>> internal;
  std::vector<int64_t> block_slot;
  std::vector<Ref> Yref, rho_psi;
  std::map<int, int64_t> ident_dim;
  std::vector<Job> recompute;  // chains of Apply with the matrices frozen (CMF)
  int64_t keep_cursor = 0;

  Ref keep(int64_t nelem) {
    Ref r{B_KEEP, keep_cursor};
    keep_cursor += align_up(nelem);
    return r;
  }
  int64_t identity_mat(int d) {
    auto it = ident_dim.find(d);
    if (it != ident_dim.end()) return it->second;
    const int64_t o = alloc_mat(d);
    P.identities.push_back({o, d});
    ident_dim[d] = o;
    return o;
  }
  // boundary key of term l at node a; -1: internal there, -2: inactive
  int bk_index(int l, int a) const {
    const int i = idx_of(l, a);
    return i < 0 ? -2 : node_bk[a][i];
  }
  std::vector<int> fkey(int l, int a, bool in) const {
    std::vector<int> k = key(l, a, in);
    return std::vector<int>(k.begin() + 2, k.end());
  }

  void comp_layout() {
    bk.assign(n, {});
    node_bk.assign(n, {});
    internal.assign(n, {});
    block_slot.assign(n, -1);
    Yref.assign(n, Ref{});
    rho_psi.assign(n, Ref{});
    for (int a = 0; a < n; ++a) {
      std::map<std::vector<int>, int> of;
      node_bk[a].assign(node_terms[a].size(), -1);
      for (size_t i = 0; i < node_terms[a].size(); ++i) {
        const int l = node_terms[a][i];
        if (is_top(a) || fkey(l, a, false).empty()) {
          internal[a].push_back(l);
          continue;
        }
        auto r = of.insert({fkey(l, a, true), (int)bk[a].size()});
        if (r.second) bk[a].push_back(BKey());
        bk[a][r.first->second].terms.push_back(l);
        node_bk[a][i] = r.first->second;
      }
      const int d = nd[a].dup();
      for (auto& b : bk[a]) {
        b.hslot = alloc_mat(d);
        b.cslot = alloc_mat(d);
        b.X = keep(nd[a].N);
      }
      if (!internal[a].empty()) {
        if (is_top(a)) {
          Yref[a] = hphi(a);
        } else {
          block_slot[a] = alloc_mat(d);
          Yref[a] = keep(nd[a].N);
        }
      }
    }
  }

  // Greedy cover of candidates by groups that agree on every leg but one.
  // sig[t][k]: object of candidate t on leg k (-1: identity); free legs from `legs`.
  std::vector<Group> cover(const std::vector<std::vector<int>>& sig, const std::vector<int>& legs) const {
    std::vector<Group> out;
    std::vector<char> done(sig.size(), 0);
    size_t left = sig.size();
    while (left > 0) {
      int best_leg = -1;
      size_t best_n = 0;
      std::vector<int> best_key;
      for (int f : legs) {
        std::map<std::vector<int>, size_t> cnt;
        for (size_t t = 0; t < sig.size(); ++t) {
          if (done[t]) continue;
          std::vector<int> k = sig[t];
          k[f] = -3;
          const size_t c = ++cnt[k];
          if (c > best_n) {
            best_n = c;
            best_leg = f;
            best_key = k;
          }
        }
      }
      Group g;
      g.free_leg = best_leg;
      for (size_t t = 0; t < sig.size(); ++t) {
        if (done[t]) continue;
        std::vector<int> k = sig[t];
        k[best_leg] = -3;
        if (k == best_key) {
          g.members.push_back((int)t);
          done[t] = 1;
          --left;
        }
      }
      out.push_back(g);
    }
    return out;
  }

  // mode products of a cover group at node a: the shared factors, and on the
  // free leg sum_l c_l H_l (a single term: its matrix scaled by c_l)
  std::vector<COp> group_ops(int a, const Group& G, const std::vector<std::vector<int>>& sig,
                             const std::vector<int>& term_of) {
    const NodeGeo& g = nd[a];
    const std::vector<int>& s0 = sig[G.members[0]];
    std::vector<COp> o;
    double2 alpha = c2(1, 0);
    for (size_t k = 0; k < g.children.size(); ++k) {
      const int c = g.children[k];
      if ((int)k != G.free_leg || G.members.size() == 1) {
        if ((int)k == G.free_leg) alpha = sop.coeff[term_of[G.members[0]]];
        if (s0[k] >= 0) o.push_back(COp{0, (int)k, mat(bk[c][s0[k]].hslot), c2(1, 0)});
        continue;
      }
      const int d = g.shape[k];
      Plan::SLin lt;
      const int64_t m = alloc_mat(d);
      lt.out = mat(m);
      lt.d = d;
      lt.first = (int)P.lin_terms.size();
      for (int t : G.members) {
        const int ob = sig[t][k];
        P.lin_terms.push_back(
            Plan::SLinTerm{sop.coeff[term_of[t]], mat(ob >= 0 ? bk[c][ob].hslot : identity_mat(d))});
      }
      lt.count = (int)G.members.size();
      P.lin.push_back(lt);
      o.push_back(COp{0, (int)k, mat(m), c2(1, 0)});
    }
    if (o.empty()) throw std::logic_error("compressed plan: a cover group without factors");
    o[0].alpha = alpha;
    return o;
  }

  // X(a,u) chain: the represent matrices of u on the children, or its leaf operators
  std::vector<COp> comp_body(int l, int a) const {
    const NodeGeo& g = nd[a];
    if (g.bottom()) return body(l, a, c2(1, 0));
    std::vector<COp> o;
    for (size_t k = 0; k < g.children.size(); ++k) {
      const int c = g.children[k];
      const int b = bk_index(l, c);
      if (b == -2) continue;
      if (b < 0) throw std::logic_error("compressed plan: internal child factor in a boundary chain");
      o.push_back(COp{0, (int)k, mat(bk[c][b].hslot), c2(1, 0)});
    }
    return o;
  }

  Job y_job(int a) {
    Job J;
    J.node = a;
    J.out = Yref[a];
    const NodeGeo& g = nd[a];
    if (g.bottom()) {
      for (int l : internal[a]) J.chains.push_back(Chain{psi(a), body(l, a, sop.coeff[l]), Ref{}});
    } else {
      for (size_t k = 0; k < g.children.size(); ++k) {
        const int c = g.children[k];
        if (block_slot[c] >= 0)
          J.chains.push_back(Chain{psi(a), {COp{0, (int)k, mat(block_slot[c]), c2(1, 0)}}, Ref{}});
      }
      std::vector<std::vector<int>> sig;
      std::vector<int> term_of;
      for (int l : internal[a]) {
        std::vector<int> s(g.children.size(), -1);
        int nact = 0;
        bool inside_one = false;
        for (size_t k = 0; k < g.children.size(); ++k) {
          const int b = bk_index(l, g.children[k]);
          if (b == -2) continue;
          ++nact;
          inside_one = inside_one || b == -1;
          s[k] = b;
        }
        if (nact < 2) continue;  // internal to one child: inside Block(child)
        if (inside_one) throw std::logic_error("compressed plan: internal child factor in a cover group");
        sig.push_back(s);
        term_of.push_back(l);
      }
      std::vector<int> legs;
      for (size_t k = 0; k < g.children.size(); ++k) legs.push_back((int)k);
      for (auto& G : cover(sig, legs)) J.chains.push_back(Chain{psi(a), group_ops(a, G, sig, term_of), Ref{}});
    }
    if (!is_top(a)) {
      J.S = mat(block_slot[a]);
      J.hp_mode = g.last();
    }
    return J;
  }

  void comp_represent() {
    int maxh = 0;
    for (auto& g : nd) maxh = std::max(maxh, g.height);
    for (int h = 0; h <= maxh; ++h) {
      std::vector<Job> jobs;
      const int64_t lin0 = (int64_t)P.lin.size();
      for (int a = 0; a < n; ++a) {
        if (nd[a].height != h) continue;
        if (!is_top(a))
          for (auto& b : bk[a]) {
            Job J;
            J.node = a;
            J.out = b.X;
            J.chains.push_back(Chain{psi(a), comp_body(b.terms[0], a), Ref{}});
            J.S = mat(b.hslot);
            J.hp_mode = nd[a].last();
            jobs.push_back(J);
          }
        if (!internal[a].empty()) jobs.push_back(y_job(a));
      }
      emit_stage(ST_LIN, lin0, (int64_t)P.lin.size(), lin0, (int64_t)P.lin.size(), "represent-sums");
      for (auto& J : jobs) {
        P.stats.rep_chains += (int64_t)J.chains.size();
        Job R = J;
        R.S = Ref{};
        recompute.push_back(R);
      }
      run_jobs(jobs, "represent");
    }
  }

  // C(a,u) for every boundary key u of a (built on the parent's tensor)
  void c_jobs(int a, std::vector<Job>& jobs, std::vector<int>& need_rho) {
    const int p = nd[a].parent;
    const NodeGeo& gp = nd[p];
    const int ia = nd[a].child_idx;
    std::vector<int> legs;
    for (size_t k = 0; k < gp.children.size(); ++k)
      if ((int)k != ia) legs.push_back((int)k);
    for (auto& b : bk[a]) {
      Job J;
      J.node = p;
      J.S = mat(b.cslot);
      J.hp_mode = ia;
      std::vector<std::vector<int>> sig;
      std::vector<int> term_of;
      std::map<int, int> wterm;  // boundary key at p -> a term with it
      for (int l : b.terms) {
        const int bp = is_top(p) ? -1 : bk_index(l, p);
        if (bp >= 0) {
          wterm.insert({bp, l});
          continue;
        }
        std::vector<int> s(gp.children.size(), -1);
        for (size_t k = 0; k < gp.children.size(); ++k) {
          if ((int)k == ia) continue;
          const int bs = bk_index(l, gp.children[k]);
          if (bs == -1) throw std::logic_error("compressed plan: internal sibling factor");
          s[k] = bs >= 0 ? bs : -1;
        }
        sig.push_back(s);
        term_of.push_back(l);
      }
      if (!sig.empty()) {
        Ref in = psi(p);
        if (!is_top(p)) {
          if (rho_psi[p].buf < 0) {
            rho_psi[p] = keep(gp.N);
            need_rho.push_back(p);
          }
          in = rho_psi[p];
        }
        for (auto& G : cover(sig, legs)) J.chains.push_back(Chain{in, group_ops(p, G, sig, term_of), Ref{}});
      }
      for (auto& kv : wterm) {
        const int l = kv.second;
        Chain ch{psi(p), {}, mat(bk[p][kv.first].cslot)};
        for (size_t k = 0; k < gp.children.size(); ++k) {
          if ((int)k == ia) continue;
          const int bs = bk_index(l, gp.children[k]);
          if (bs >= 0) ch.ops.push_back(COp{0, (int)k, mat(bk[gp.children[k]][bs].hslot), c2(1, 0)});
        }
        J.chains.push_back(ch);
      }
      if (J.chains.size() == 1 && J.chains[0].H.buf >= 0) {  // one chain: its last factor is a mode product
        J.chains[0].ops.push_back(COp{0, gp.last(), J.chains[0].H, c2(1, 0)});
        J.chains[0].H = Ref{};
      }
      jobs.push_back(J);
    }
  }

  void comp_meanfield() {
    int maxdepth = 0;
    for (auto& g : nd) maxdepth = std::max(maxdepth, g.depth);
    for (int d = 1; d <= maxdepth; ++d) {
      std::vector<Job> jobs;
      std::vector<int> need_rho;
      const int64_t lin0 = (int64_t)P.lin.size();
      for (int a = 0; a < n; ++a)
        if (nd[a].depth == d) c_jobs(a, jobs, need_rho);
      std::vector<Job> rj;
      for (int p : need_rho) {
        Job J;
        J.node = p;
        J.out = rho_psi[p];
        J.chains.push_back(Chain{psi(p), {COp{0, nd[p].last(), mat(P.rho_off[p]), c2(1, 0)}}, Ref{}});
        rj.push_back(J);
      }
      run_jobs(rj, "meanfield-rho");
      emit_stage(ST_LIN, lin0, (int64_t)P.lin.size(), lin0, (int64_t)P.lin.size(), "meanfield-sums");
      for (auto& J : jobs) P.stats.mf_chains += (int64_t)J.chains.size();
      run_jobs(jobs, "meanfield");
    }
  }

  void comp_apply(bool fused = false) {
    std::vector<Job> jobs;
    std::vector<char> started(n, 0);
    for (int a = 0; a < n; ++a) {
      if (is_top(a)) {
        started[a] = internal[a].empty() ? 0 : 1;  // Y(top) is H Phi_top
        continue;
      }
      if (fused) {  // the derivative accumulates the kept chains directly
        started[a] = 1;
        continue;
      }
      if (internal[a].empty() && bk[a].empty()) continue;
      Job J;
      J.node = a;
      J.out = hphi(a);
      if (!internal[a].empty()) J.chains.push_back(Chain{Yref[a], {}, mat(P.rho_off[a])});
      for (auto& b : bk[a]) J.chains.push_back(Chain{b.X, {}, mat(b.cslot)});
      P.stats.app_chains += (int64_t)J.chains.size();
      jobs.push_back(J);
      started[a] = 1;
    }
    run_jobs(jobs, "apply");
    int64_t t0 = (int64_t)P.acc.size(), tile0 = (int64_t)P.acc_tiles.size();
    for (int a = 0; a < n; ++a)
      if (!started[a]) add_acc(hphi(a), false, c2(1.0, 0.0), a, {}, false);
    emit_stage(ST_ACC, t0, (int64_t)P.acc.size(), tile0, (int64_t)P.acc_tiles.size(), "apply-zero");
  }

  static bool single_plain(const Job& J) { return J.chains.size() == 1 && J.chains[0].H.buf < 0; }
  static bool needs_sum(const Job& J) {
    return !single_plain(J) || (J.chains[0].ops.empty() && J.out.buf >= 0);
  }

  // Run independent jobs: per scratch chunk one stage per mode-product
  // position, one accumulation stage for the sums, one hole-product stage.
  void run_jobs(std::vector<Job>& jobs, const char* name) {
    size_t i = 0;
    while (i < jobs.size()) {
      int64_t cursor = 0;
      size_t j = i;
      std::vector<std::vector<std::pair<int64_t, int64_t>>> cb;
      std::vector<int64_t> tmp;
      while (j < jobs.size()) {
        const Job& J = jobs[j];
        const int64_t Na = align_up(nd[J.node].N);
        int64_t need = 0;
        std::vector<std::pair<int64_t, int64_t>> b;
        for (auto& ch : J.chains) {
          const int nb = (int)std::min<size_t>(2, ch.ops.size());
          b.push_back({nb > 0 ? cursor + need : -1, nb > 1 ? cursor + need + Na : -1});
          need += nb * Na;
        }
        int64_t t = -1;
        if (needs_sum(J) && J.out.buf < 0) {
          t = cursor + need;
          need += Na;
        }
        if (j > i && cursor + need > budget) break;
        cursor += need;
        cb.push_back(b);
        tmp.push_back(t);
        ++j;
      }
      P.scratch_size = std::max(P.scratch_size, cursor);
      auto result = [&](size_t k, size_t c) -> Ref {
        const Job& J = jobs[k];
        const Chain& ch = J.chains[c];
        const size_t no = ch.ops.size();
        if (no == 0) return ch.in;
        if (single_plain(J) && J.out.buf >= 0) return J.out;
        const auto& b = cb[k - i][c];
        return Ref{B_SCR, (no - 1) % 2 == 0 ? b.first : b.second};
      };
      auto final_ref = [&](size_t k) -> Ref {
        const Job& J = jobs[k];
        if (!needs_sum(J)) return result(k, 0);
        return J.out.buf >= 0 ? J.out : Ref{B_SCR, tmp[k - i]};
      };
      size_t maxops = 0;
      for (size_t k = i; k < j; ++k)
        for (auto& ch : jobs[k].chains) maxops = std::max(maxops, ch.ops.size());
      for (size_t pos = 0; pos < maxops; ++pos) {
        const int64_t t0 = (int64_t)P.mp.size(), tile0 = (int64_t)P.mp_tiles.size();
        for (size_t k = i; k < j; ++k) {
          const Job& J = jobs[k];
          for (size_t c = 0; c < J.chains.size(); ++c) {
            const Chain& ch = J.chains[c];
            if (pos >= ch.ops.size()) continue;
            const auto& b = cb[k - i][c];
            const Ref in = pos == 0 ? ch.in : Ref{B_SCR, (pos - 1) % 2 == 0 ? b.first : b.second};
            const Ref out = pos + 1 == ch.ops.size() ? result(k, c) : Ref{B_SCR, pos % 2 == 0 ? b.first : b.second};
            const COp& op = ch.ops[pos];
            add_mp(in, out, op.mat, op.alpha, J.node, op.mode, op.kind == 1);
          }
        }
        emit_stage(ST_MP, t0, (int64_t)P.mp.size(), tile0, (int64_t)P.mp_tiles.size(), name);
      }
      {
        const int64_t t0 = (int64_t)P.acc.size(), tile0 = (int64_t)P.acc_tiles.size();
        for (size_t k = i; k < j; ++k) {
          const Job& J = jobs[k];
          if (!needs_sum(J)) continue;
          std::vector<Plan::SAccTerm> terms;
          for (size_t c = 0; c < J.chains.size(); ++c) terms.push_back(Plan::SAccTerm{J.chains[c].H, result(k, c)});
          add_acc(final_ref(k), false, c2(1.0, 0.0), J.node, terms, false);
        }
        emit_stage(ST_ACC, t0, (int64_t)P.acc.size(), tile0, (int64_t)P.acc_tiles.size(), name);
      }
      {
        const int64_t t0 = (int64_t)P.hp.size(), tile0 = (int64_t)P.hp_tiles.size();
        for (size_t k = i; k < j; ++k) {
          const Job& J = jobs[k];
          if (J.S.buf < 0) continue;
          add_hp(psi(J.node), final_ref(k), J.S, J.node, J.hp_mode);
        }
        emit_stage(ST_HP, t0, (int64_t)P.hp.size(), tile0, (int64_t)P.hp_tiles.size(), name);
      }
      i = j;
    }
  }

  // Apply and LayerDerivative with every matrix frozen (constant-mean-field
  // steps): the kept chains are recomputed from the current Phi.
  void comp_frozen_apply() {
    run_jobs(recompute, "apply-chains");
    comp_apply();
    stage_final();
  }


  // ---- environment of the energy gradient, compressed plan -----------------
  // E_out[a], the mean field of the terms acting only outside a, built at
  // the parent p like the grouped plan's stage_environment: terms internal to
  // p that miss a (Block of every sibling, LCA-p cover groups over the other
  // siblings) on Phi_p x_last rho_p, boundary restrictions w of p that miss a
  // with C(p,w) on the parent index, and E_out[p] on the parent index.
  void comp_environment() {
    eout_off.assign(n, -1);
    std::vector<char> rho_done(n, 0);
    for (int p = 0; p < n; ++p) rho_done[p] = rho_psi[p].buf >= 0;  // computed in comp_meanfield
    int maxdepth = 0;
    for (auto& g : nd) maxdepth = std::max(maxdepth, g.depth);
    for (int dep = 1; dep <= maxdepth; ++dep) {
      std::vector<Job> rj, jobs;
      const int64_t lin0 = (int64_t)P.lin.size();
      for (int a = 0; a < n; ++a) {
        if (nd[a].depth != dep) continue;
        const int p = nd[a].parent;
        const NodeGeo& gp = nd[p];
        const int ia = nd[a].child_idx;
        eout_off[a] = alloc_mat(nd[a].dup());
        Ref in_rho = psi(p);
        if (!is_top(p)) {
          if (rho_psi[p].buf < 0) rho_psi[p] = keep(gp.N);
          if (!rho_done[p]) {
            Job R;
            R.node = p;
            R.out = rho_psi[p];
            R.chains.push_back(Chain{psi(p), {COp{0, gp.last(), mat(P.rho_off[p]), c2(1, 0)}}, Ref{}});
            rj.push_back(R);
            rho_done[p] = 1;
          }
          in_rho = rho_psi[p];
        }
        Job J;
        J.node = p;
        J.S = mat(eout_off[a]);
        J.hp_mode = ia;
        for (size_t k = 0; k < gp.children.size(); ++k) {
          const int c = gp.children[k];
          if ((int)k == ia || block_slot[c] < 0) continue;
          J.chains.push_back(Chain{in_rho, {COp{0, (int)k, mat(block_slot[c]), c2(1, 0)}}, Ref{}});
        }
        std::vector<std::vector<int>> sig;
        std::vector<int> term_of;
        lca_terms(p, ia, sig, term_of);
        std::vector<int> legs;
        for (size_t k = 0; k < gp.children.size(); ++k)
          if ((int)k != ia) legs.push_back((int)k);
        for (auto& G : cover(sig, legs)) J.chains.push_back(Chain{in_rho, group_ops(p, G, sig, term_of), Ref{}});
        if (!is_top(p)) {
          for (auto& b : bk[p]) {
            const int l = b.terms[0];
            if (bk_index(l, a) != -2) continue;  // the restriction touches a
            Chain ch{psi(p), {}, mat(b.cslot)};
            for (size_t k = 0; k < gp.children.size(); ++k) {
              const int bs = bk_index(l, gp.children[k]);
              if (bs >= 0) ch.ops.push_back(COp{0, (int)k, mat(bk[gp.children[k]][bs].hslot), c2(1, 0)});
            }
            J.chains.push_back(ch);
          }
          J.chains.push_back(Chain{psi(p), {}, mat(eout_off[p])});
        }
        if (J.chains.empty()) J.chains.push_back(Chain{psi(p), {}, mat(zero_mat(gp.dup()))});
        jobs.push_back(J);
      }
      run_jobs(rj, "environment-rho");
      emit_stage(ST_LIN, lin0, (int64_t)P.lin.size(), lin0, (int64_t)P.lin.size(), "environment-sums");
      run_jobs(jobs, "environment");
    }
  }

  // ---- SCF sweep segments (QT_PLAN_SCF) ------------------------------------
  // HamiltonianRepresentation(H, tree, tree, tail=false) of the SCF
  // (src/Applications/SCF.cpp:267-341): every term's sparse tree ends at the
  // lowest common ancestor (LCA) of its leaves.  Per node, on top of the
  // compressed objects (H(a,u), Block(a) = hCorr[a]):
  //   O_a      hole overlap <Phi_p|Phi_p> at a: the hole matrix of every term
  //            whose LCA is a (its parent lies outside the term's tree)
  //   C'(a,u)  sum_l c_l hCons_l(a) of the boundary terms with restriction u;
  //            built at p from the sibling matrices on Phi_p x_last O_p (LCA = p)
  //            and from C'(p,w) (LCA above p)
  //   Eout(a)  hConCorr[a]: terms acting only outside a
  //            (buildDownCorrection, src/TreeClasses/HamiltonianRepresentation.cpp:163-203)
  // buildUp(a) = the compressed represent jobs of a; buildDown(a) = O_a,
  // C'(a,.), Eout(a); the effective Hamiltonian of SCF.cpp:36-84 is
  //   H_eff(a) A = [LCA-a terms on A] x_last O_a + sum_k Block(k) x_k A
  //              + sum_u (u on A) x_last C'(a,u) + A x_last Eout(a).
  std::vector<std::vector<int64_t>> scf_c;  // C'(a,u) slots
  std::vector<int64_t> o_slot, eout_slot;
  std::vector<Ref> o_psi;  // Phi_p x_last O_p
  std::map<int, int64_t> zero_dim;

  int64_t zero_mat(int d) {
    auto it = zero_dim.find(d);
    if (it != zero_dim.end()) return it->second;
    const int64_t o = alloc_mat(d);  // B_MATS is zeroed once at prepare and never written here
    zero_dim[d] = o;
    return o;
  }

  // LCA-a terms of node a: internal terms that touch two or more children
  // (their signatures over the child legs for the cover)
  void lca_terms(int a, int skip_child, std::vector<std::vector<int>>& sig, std::vector<int>& term_of) {
    const NodeGeo& g = nd[a];
    for (int l : internal[a]) {
      if (g.bottom()) continue;
      std::vector<int> s(g.children.size(), -1);
      int nact = 0;
      bool touches_skip = false, inside_one = false;
      for (size_t k = 0; k < g.children.size(); ++k) {
        const int b = bk_index(l, g.children[k]);
        if (b == -2) continue;
        ++nact;
        if ((int)k == skip_child) touches_skip = true;
        inside_one = inside_one || b == -1;
        s[k] = b;
      }
      if (nact < 2 || touches_skip) continue;
      if (inside_one) throw std::logic_error("SCF plan: internal child factor in an LCA term");
      sig.push_back(s);
      term_of.push_back(l);
    }
  }

  void scf_segments() {
    P.scf = true;
    scf_c.assign(n, {});
    o_slot.assign(n, -1);
    eout_slot.assign(n, -1);
    o_psi.assign(n, Ref{});
    int64_t maxN = 16;
    for (int a = 0; a < n; ++a) {
      maxN = std::max(maxN, nd[a].N);
      const int d = nd[a].dup();
      for (size_t u = 0; u < bk[a].size(); ++u) scf_c[a].push_back(alloc_mat(d));
      if (!is_top(a)) {
        o_slot[a] = alloc_mat(d);
        eout_slot[a] = alloc_mat(d);
      }
      if (!is_top(a) && !nd[a].bottom()) o_psi[a] = keep(nd[a].N);
    }
    P.kry_in = 0;
    P.kry_out = align_up(maxN);
    P.kry_size = 2 * align_up(maxN);
    const Ref kin{B_KRY, P.kry_in}, kout{B_KRY, P.kry_out};
    P.scf_up_b.assign(n, 0);
    P.scf_up_e.assign(n, 0);
    P.scf_down_b.assign(n, 0);
    P.scf_down_e.assign(n, 0);
    P.scf_apply_b.assign(n, 0);
    P.scf_apply_e.assign(n, 0);
    for (int a = 0; a < n; ++a) {
      const NodeGeo& g = nd[a];
      // buildUp(a)
      P.scf_up_b[a] = (int64_t)P.stages.size();
      if (!is_top(a)) {
        std::vector<Job> jobs;
        const int64_t lin0 = (int64_t)P.lin.size();
        for (auto& b : bk[a]) {
          Job J;
          J.node = a;
          J.out = b.X;
          J.chains.push_back(Chain{psi(a), comp_body(b.terms[0], a), Ref{}});
          J.S = mat(b.hslot);
          J.hp_mode = g.last();
          jobs.push_back(J);
        }
        if (!internal[a].empty()) jobs.push_back(y_job(a));
        emit_stage(ST_LIN, lin0, (int64_t)P.lin.size(), lin0, (int64_t)P.lin.size(), "scf-up-sums");
        run_jobs(jobs, "scf-up");
      }
      P.scf_up_e[a] = (int64_t)P.stages.size();
      // buildDown(a)
      P.scf_down_b[a] = (int64_t)P.stages.size();
      if (!is_top(a)) scf_down(a);
      P.scf_down_e[a] = (int64_t)P.stages.size();
      // effective Hamiltonian at a
      P.scf_apply_b[a] = (int64_t)P.stages.size();
      {
        const int64_t lin0 = (int64_t)P.lin.size();
        Job J;
        J.node = a;
        J.out = kout;
        const Ref oa = is_top(a) ? Ref{} : mat(o_slot[a]);
        if (g.bottom()) {
          for (int l : internal[a]) J.chains.push_back(Chain{kin, body(l, a, sop.coeff[l]), oa});
        } else {
          std::vector<std::vector<int>> sig;
          std::vector<int> term_of;
          lca_terms(a, -1, sig, term_of);
          std::vector<int> legs;
          for (size_t k = 0; k < g.children.size(); ++k) legs.push_back((int)k);
          for (auto& G : cover(sig, legs)) J.chains.push_back(Chain{kin, group_ops(a, G, sig, term_of), oa});
          for (size_t k = 0; k < g.children.size(); ++k) {
            const int c = g.children[k];
            if (block_slot[c] >= 0)
              J.chains.push_back(Chain{kin, {COp{0, (int)k, mat(block_slot[c]), c2(1, 0)}}, Ref{}});
          }
        }
        for (size_t u = 0; u < bk[a].size(); ++u)
          J.chains.push_back(Chain{kin, comp_body(bk[a][u].terms[0], a), mat(scf_c[a][u])});
        if (!is_top(a)) J.chains.push_back(Chain{kin, {}, mat(eout_slot[a])});
        if (J.chains.empty()) J.chains.push_back(Chain{kin, {}, mat(zero_mat(g.dup()))});
        emit_stage(ST_LIN, lin0, (int64_t)P.lin.size(), lin0, (int64_t)P.lin.size(), "scf-apply-sums");
        std::vector<Job> jobs{J};
        run_jobs(jobs, "scf-apply");
      }
      P.scf_apply_e[a] = (int64_t)P.stages.size();
    }
  }

  void scf_down(int a) {
    const int p = nd[a].parent;
    const NodeGeo& gp = nd[p];
    const int ia = nd[a].child_idx;
    // O_a = <Phi_p|Phi_p> with the hole at a, and Phi_p x_last O_p
    {
      std::vector<Job> jobs;
      Job J;
      J.node = p;
      J.chains.push_back(Chain{psi(p), {}, Ref{}});
      J.S = mat(o_slot[a]);
      J.hp_mode = ia;
      jobs.push_back(J);
      if (!is_top(p)) {
        Job R;
        R.node = p;
        R.out = o_psi[p];
        R.chains.push_back(Chain{psi(p), {COp{0, gp.last(), mat(o_slot[p]), c2(1, 0)}}, Ref{}});
        jobs.push_back(R);
      }
      run_jobs(jobs, "scf-down-overlap");
    }
    const Ref in_lca = is_top(p) ? psi(p) : o_psi[p];
    std::vector<int> legs;
    for (size_t k = 0; k < gp.children.size(); ++k)
      if ((int)k != ia) legs.push_back((int)k);
    std::vector<Job> jobs;
    const int64_t lin0 = (int64_t)P.lin.size();
    // C'(a,u)
    for (size_t u = 0; u < bk[a].size(); ++u) {
      Job J;
      J.node = p;
      J.S = mat(scf_c[a][u]);
      J.hp_mode = ia;
      std::vector<std::vector<int>> sig;
      std::vector<int> term_of;
      std::map<int, int> wterm;
      for (int l : bk[a][u].terms) {
        const int bp = is_top(p) ? -1 : bk_index(l, p);
        if (bp >= 0) {
          wterm.insert({bp, l});
          continue;
        }
        std::vector<int> sg(gp.children.size(), -1);
        for (size_t k = 0; k < gp.children.size(); ++k) {
          if ((int)k == ia) continue;
          const int bs = bk_index(l, gp.children[k]);
          if (bs == -1) throw std::logic_error("SCF plan: internal sibling factor");
          sg[k] = bs >= 0 ? bs : -1;
        }
        sig.push_back(sg);
        term_of.push_back(l);
      }
      for (auto& G : cover(sig, legs)) J.chains.push_back(Chain{in_lca, group_ops(p, G, sig, term_of), Ref{}});
      for (auto& kv : wterm) {
        Chain ch{psi(p), {}, mat(scf_c[p][kv.first])};
        for (size_t k = 0; k < gp.children.size(); ++k) {
          if ((int)k == ia) continue;
          const int bs = bk_index(kv.second, gp.children[k]);
          if (bs >= 0) ch.ops.push_back(COp{0, (int)k, mat(bk[gp.children[k]][bs].hslot), c2(1, 0)});
        }
        J.chains.push_back(ch);
      }
      jobs.push_back(J);
    }
    // Eout(a)
    {
      Job J;
      J.node = p;
      J.S = mat(eout_slot[a]);
      J.hp_mode = ia;
      std::vector<std::vector<int>> sig;
      std::vector<int> term_of;
      lca_terms(p, ia, sig, term_of);
      for (auto& G : cover(sig, legs)) J.chains.push_back(Chain{in_lca, group_ops(p, G, sig, term_of), Ref{}});
      if (!is_top(p))
        for (size_t w = 0; w < bk[p].size(); ++w) {
          const int l = bk[p][w].terms[0];
          if (bk_index(l, a) != -2) continue;  // the restriction w touches a
          Chain ch{psi(p), {}, mat(scf_c[p][w])};
          for (size_t k = 0; k < gp.children.size(); ++k) {
            const int bs = bk_index(l, gp.children[k]);
            if (bs >= 0) ch.ops.push_back(COp{0, (int)k, mat(bk[gp.children[k]][bs].hslot), c2(1, 0)});
          }
          J.chains.push_back(ch);
        }
      for (size_t k = 0; k < gp.children.size(); ++k) {
        const int c = gp.children[k];
        if ((int)k == ia || block_slot[c] < 0) continue;
        J.chains.push_back(Chain{psi(p), {COp{0, (int)k, mat(block_slot[c]), c2(1, 0)}}, Ref{}});
      }
      if (!is_top(p)) J.chains.push_back(Chain{psi(p), {}, mat(eout_slot[p])});
      if (J.chains.empty()) J.chains.push_back(Chain{psi(p), {}, mat(zero_mat(gp.dup()))});
      jobs.push_back(J);
    }
    emit_stage(ST_LIN, lin0, (int64_t)P.lin.size(), lin0, (int64_t)P.lin.size(), "scf-down-sums");
    run_jobs(jobs, "scf-down");
  }

  // Flops of the reference call sequence (independent of this plan):
  // mode product 8*N*a, hole product 8*N*a, diagonal leaf op 6*N, complex
  // scale 6*N, accumulate 2*N, projector 24*N*d + 2*N, rho^-1 8*N*d.
  void count_reference_flops() {
    double F = 0;
    for (int a = 0; a < n; ++a) {
      if (is_top(a)) continue;
      const NodeGeo& p = nd[nd[a].parent];
      F += 8.0 * p.N * p.dup() + 8.0 * p.N * nd[a].dup();
    }
    auto body_flops = [&](int l, int a) {
      const NodeGeo& g = nd[a];
      double f = 0;
      if (g.bottom()) {
        for (int x = sop.ptr[l]; x < sop.ptr[l + 1]; ++x)
          if (sop.mode[x] == g.leaf_mode) f += ops.kind[sop.op[x]] == 0 ? 8.0 * g.N * g.shape[0] : 6.0 * g.N;
      } else {
        for (size_t k = 0; k < g.children.size(); ++k)
          if (act(l, g.children[k])) f += 8.0 * g.N * g.shape[k];
      }
      return f;
    };
    for (int l = 0; l < L; ++l)
      for (int a : term_nodes[l]) {
        const NodeGeo& g = nd[a];
        double app = 6.0 * g.N + body_flops(l, a) + (is_top(a) ? 2.0 * g.N : 8.0 * g.N * g.dup() + 2.0 * g.N);
        F += app;
        if (is_top(a)) {
          F += app;  // Expectation repeats Apply at the top
          continue;
        }
        F += body_flops(l, a) + 8.0 * g.N * g.dup();  // represent
        const NodeGeo& p = nd[g.parent];
        for (size_t k = 0; k < p.children.size(); ++k)
          if ((int)k != g.child_idx && act(l, p.children[k])) F += 8.0 * p.N * p.shape[k];
        if (!p.top()) F += 8.0 * p.N * p.dup();
        F += 8.0 * p.N * g.dup();  // mean field
      }
    for (int a = 0; a < n; ++a) {
      const NodeGeo& g = nd[a];
      if (is_top(a)) {
        F += 6.0 * g.N + 8.0 * g.N * g.dup();
      } else {
        F += 24.0 * g.N * g.dup() + 2.0 * g.N + 8.0 * g.N * g.dup() + 6.0 * g.N;
      }
    }
    P.stats.ref_flops = F;
  }
};

}  // namespace

std::string build_plan(Plan& plan, const std::vector<NodeGeo>& nodes, const OpTable& ops,
                       const SopDesc& sop, int flavour, int prec, int64_t scratch_budget_elems,
                       bool grad, const CdvrDesc* cdvr, const TcTune& tune) {
  plan = Plan();
  plan.want_grad = grad;
  plan.tune = tune;
  try {
    if (prec < 0 || prec > 2) throw std::runtime_error("unknown precision");
    const bool scf = (flavour & 0x2000) != 0;
    if (cdvr) {
      if ((flavour & ~0xA000) == 2) throw std::runtime_error("the CDVR potential needs the reference or grouped plan");
      if (prec != 0) throw std::runtime_error("the CDVR potential runs in complex128 arithmetic");
      if (scf) throw std::runtime_error("the SCF sweep has no CDVR potential (nor has the reference's)");
      if (grad) throw std::runtime_error("no energy gradient with the CDVR potential");
    }
    if ((flavour & 0x8000) && prec == 0)
      throw std::runtime_error("tensor-core mode products need double-float or complex64 arithmetic");
    plan.mp_tensor = (flavour & 0x8000) != 0;
    plan.hp_tensor = plan.mp_tensor && prec == 1;
    Builder b(plan, nodes, ops, sop, flavour & ~0xA000, prec, scratch_budget_elems);
    b.set_scf(scf);
    b.set_cdvr(cdvr);
    b.run();
  } catch (const std::exception& e) {
    return e.what();
  }
  plan.ops_size = (int64_t)ops.data.size() / 2;
  return "";
}

}  // namespace qt
