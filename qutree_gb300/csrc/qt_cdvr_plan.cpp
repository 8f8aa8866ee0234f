// qt_cdvr_plan.cpp -- stages of the CDVR potential (Hamiltonians with a
// non-SOP potential, H.hasV) for the reference and grouped sweep plans.
//
// CDVR::Update (src/DVR/CDVR.cpp:150-175) runs inside the build part of the
// sweep (after the density matrices and the mean fields), CDVR::apply
// (src/DVR/CDVR.cpp:90-123) inside the Apply part: its result is added to
// H Phi before the projector and the inverse density, as Apply does
// (src/TreeClasses/HamiltonianRepresentation.cpp:30-32).  Everything lives
// in B_CDVR; the contractions are strided-contraction tasks (ST_TC).
//
// Update, in stage order:
//   Chi = gramSchmidt(Psi + seeded noise)           Regularize, src/DVR/XMatrixTrees.cpp:6-19
//   rho(Chi), its inverse square root (eps 1e-8)     XMatrixTrees::UnweightContractions
//   X matrices on the leaf-to-root paths             represent(mats_, Xsop, Psi, Psi)
//   X holes (tail-free inverse trees), weighted      contraction(holes_, Chi, Chi, mats_, rho)
//   grids: one matrix -> eigenvectors, several ->    LayerGrid, src/DVR/TDDVR.cpp:63-89
//     weighted simultaneous diagonalisation
//   sqrt(rho), its regularised inverse (eps 1e-7)    MatrixTensorTree::buildEdges
//   node tensors to the grids, edges                 TDDVR::GridTransformation
//   bottom-up / top-down normalised coefficients     MatrixTensorTree::{bottomUp,topDown}Normalized
//   V on node and edge grids                         UpdateNodeDVR / UpdateEdgeDVR
//   correction tensors, bottom-up                    calculateDeltaVs, src/DVR/cdvr_functions.cpp:67-215
// MatrixTensorTree starts from orthogonal(Psi); on the orthonormal Psi every
// sweep requires that is the identity up to rounding and is not formed.
#include <algorithm>
#include <random>
#include <stdexcept>

#include "qt_internal.h"

namespace qt {
namespace {

constexpr int64_t kAl = 16;
int64_t al(int64_t x) { return (x + kAl - 1) / kAl * kAl; }
double2 cx(double r, double i = 0.0) {
  double2 v;
  v.x = r;
  v.y = i;
  return v;
}

class CdvrBuilder {
 public:
  CdvrBuilder(Plan& P, const CdvrDesc& D) : P(P), nd(P.nodes), D(D), L(P.cd) { derive(); }

  double update() {
    layout();
    P.cdvr_update_begin = (int64_t)P.stages.size();
    st_chi();
    st_rho_chi();
    st_xmats();
    st_xholes();
    st_grids();
    st_edges();
    st_potential();
    st_delta_v();
    P.cdvr_update_end = (int64_t)P.stages.size();
    return flops;
  }

  double apply() {
    st_apply();
    return flops;
  }

 private:
  Plan& P;
  std::vector<NodeGeo>& nd;
  const CdvrDesc& D;
  Plan::CdvrLayout& L;
  int n = 0, f = 0;
  int64_t cur = 0;
  double flops = 0;
  std::vector<int> leaf_node;            // mode -> bottom node
  std::vector<std::vector<int>> sub;     // node -> modes of its subtree (ascending)
  std::vector<std::vector<int>> path;    // mode -> nodes from its bottom node up to the top

  Ref cd(int64_t off) const { return Ref{B_CDVR, off}; }
  Ref psi(int a) const { return Ref{B_PSI, nd[a].aoff}; }
  Ref hphi(int a) const { return Ref{B_HPHI, nd[a].aoff}; }
  Ref mat(int64_t off) const { return Ref{B_MATS, off}; }
  int64_t take(int64_t elems) {
    const int64_t o = cur;
    cur += al(std::max<int64_t>(elems, 1));
    return o;
  }
  bool top(int a) const { return nd[a].parent < 0; }
  bool in_sub(int a, int m) const { return std::binary_search(sub[a].begin(), sub[a].end(), m); }

  // ---- task constructors -------------------------------------------------
  void tc_push(const Plan::STC& t) {
    const int task = (int)P.tc.size();
    P.tc.push_back(t);
    const int64_t M = (int64_t)t.M0 * t.M1, N = (int64_t)t.N0 * t.N1;
    for (int64_t mt = 0; mt < M; mt += kTcTile)
      for (int64_t nt = 0; nt < N; nt += kTcTile)
        P.tc_tiles.push_back(make_int4(task, (int)(mt / kTcTile), (int)(nt / kTcTile), 0));
    flops += 8.0 * (double)M * N * t.K0 * t.K1;
  }
  static Plan::STC tc0() {
    Plan::STC t{};
    t.alpha = cx(1.0);
    t.M0 = t.M1 = t.N0 = t.N1 = t.K0 = t.K1 = 1;
    return t;
  }
  // out = op(h) x_k in on a tensor of shape dims; op: 'N', 'T', 'H' (adjoint), 'C' (conjugate)
  void tc_mode(Ref in, Ref out, Ref h, const std::vector<int>& dims, int k, char op, bool add) {
    int64_t before = 1, after = 1;
    for (int i = 0; i < k; ++i) before *= dims[i];
    for (size_t i = k + 1; i < dims.size(); ++i) after *= dims[i];
    const int d = dims[k];
    Plan::STC t = tc0();
    t.A = in;
    t.B = h;
    t.C = out;
    t.M0 = (int)before;
    t.M1 = (int)after;
    t.am0 = 1;
    t.am1 = before * d;
    t.K0 = d;
    t.ak0 = before;
    t.N0 = d;
    if (op == 'N' || op == 'C') {
      t.bk0 = d;
      t.bn0 = 1;
    } else {
      t.bk0 = 1;
      t.bn0 = d;
    }
    t.conjB = (op == 'H' || op == 'C') ? 1 : 0;
    t.cm0 = 1;
    t.cm1 = before * d;
    t.cn0 = before;
    t.add = add ? 1 : 0;
    tc_push(t);
  }
  // S(i, j) = sum over all indices but k of conj(A[.. i ..]) B[.. j ..]
  void tc_hole(Ref S, Ref A, Ref B, const std::vector<int>& dims, int k) {
    int64_t before = 1, after = 1;
    for (int i = 0; i < k; ++i) before *= dims[i];
    for (size_t i = k + 1; i < dims.size(); ++i) after *= dims[i];
    const int d = dims[k];
    Plan::STC t = tc0();
    t.A = A;
    t.B = B;
    t.C = S;
    t.M0 = d;
    t.am0 = before;
    t.K0 = (int)before;
    t.ak0 = 1;
    t.K1 = (int)after;
    t.ak1 = before * d;
    t.conjA = 1;
    t.bk0 = 1;
    t.bk1 = before * d;
    t.N0 = d;
    t.bn0 = before;
    t.cm0 = 1;
    t.cn0 = d;
    tc_push(t);
  }
  // C = opA(A) opB(B), d x d; op 'N', 'H' (adjoint), 'C' (conjugate)
  void tc_mm(Ref C, Ref A, char opA, Ref B, char opB, int d) {
    Plan::STC t = tc0();
    t.A = A;
    t.B = B;
    t.C = C;
    t.M0 = t.N0 = t.K0 = d;
    if (opA == 'H') {
      t.am0 = d;
      t.ak0 = 1;
    } else {
      t.am0 = 1;
      t.ak0 = d;
    }
    t.conjA = opA != 'N';
    if (opB == 'H') {
      t.bk0 = d;
      t.bn0 = 1;
    } else {
      t.bk0 = 1;
      t.bn0 = d;
    }
    t.conjB = opB != 'N';
    t.cm0 = 1;
    t.cn0 = d;
    tc_push(t);
  }

  std::vector<int> shape(int a) const { return nd[a].shape; }
  int dup(int a) const { return nd[a].dup(); }

  void emit(int kind, int64_t t0, int64_t t1, int64_t tile0, int64_t tile1, const char* name,
            double fl) {
    if (t1 <= t0) return;
    Stage s;
    s.kind = kind;
    s.first_task = t0;
    s.n_tasks = t1 - t0;
    s.first_tile = tile0;
    s.n_tiles = tile1 - tile0;
    s.name = name;
    s.flops = fl;
    P.stages.push_back(s);
  }
  // brackets a group of strided-contraction tasks as one stage
  struct TcMark {
    int64_t t0, tile0;
    double f0;
  };
  TcMark tc_begin() const { return TcMark{(int64_t)P.tc.size(), (int64_t)P.tc_tiles.size(), flops}; }
  void tc_end(const TcMark& m, const char* name) {
    emit(ST_TC, m.t0, (int64_t)P.tc.size(), m.tile0, (int64_t)P.tc_tiles.size(), name, flops - m.f0);
  }

  // ---- tree structure ----------------------------------------------------
  void derive() {
    n = (int)nd.size();
    f = (int)D.leaf_x.size();
    if (f > 256) throw std::runtime_error("CDVR: more than 256 modes");
    int roots = 0;
    for (int a = 0; a < n; ++a) roots += top(a) ? 1 : 0;
    if (roots != 1) throw std::runtime_error("CDVR needs a single tree");
    leaf_node.assign(f, -1);
    for (int a = 0; a < n; ++a)
      if (nd[a].bottom()) {
        const int m = nd[a].leaf_mode;
        if (m < 0 || m >= f) throw std::runtime_error("CDVR: leaf grids do not cover the modes");
        leaf_node[m] = a;
        if ((int)D.leaf_x[m].size() != nd[a].shape[0])
          throw std::runtime_error("CDVR: leaf grid size differs from the leaf dimension");
      }
    for (int m = 0; m < f; ++m)
      if (leaf_node[m] < 0) throw std::runtime_error("CDVR: a leaf grid without a leaf");
    for (int a = 0; a < n; ++a)
      if ((int)nd[a].shape.size() > 6) throw std::runtime_error("CDVR: node order above 6");
    sub.assign(n, {});
    path.assign(f, {});
    for (int m = 0; m < f; ++m) {
      int a = leaf_node[m];
      while (a >= 0) {
        path[m].push_back(a);
        sub[a].push_back(m);
        a = nd[a].parent;
      }
    }
    for (auto& s : sub) std::sort(s.begin(), s.end());
    if (nd[P.tops[0]].bottom()) throw std::runtime_error("CDVR needs a tree with more than one node");
  }

  // ---- layout ------------------------------------------------------------
  void layout() {
    cur = 0;
    auto per_node = [&](std::vector<int64_t>& v, bool non_top, bool parent_size) {
      v.assign(n, -1);
      for (int a = 0; a < n; ++a) {
        if (non_top && top(a)) continue;
        v[a] = take(parent_size ? nd[nd[a].parent].N : nd[a].N);
      }
    };
    auto per_mat = [&](std::vector<int64_t>& v, bool non_top) {
      v.assign(n, -1);
      for (int a = 0; a < n; ++a) {
        if (non_top && top(a)) continue;
        v[a] = take((int64_t)dup(a) * dup(a));
      }
    };
    per_node(L.noise, false, false);
    per_node(L.chi, false, false);
    per_node(L.at, false, false);
    per_node(L.cup, true, false);
    L.cup[P.tops[0]] = L.at[P.tops[0]];
    per_node(L.cdown, true, true);
    per_node(L.vnode, false, false);
    per_node(L.xi, false, false);
    per_node(L.vx, false, false);
    per_node(L.tmpa, false, false);
    per_node(L.tmpb, false, false);
    per_mat(L.rho_chi, false);
    per_mat(L.isq, true);
    per_mat(L.trafo, true);
    per_mat(L.htrafo, true);
    per_mat(L.sqrt_rho, true);
    per_mat(L.binv, true);
    per_mat(L.g, true);
    per_mat(L.sqrho, true);
    per_mat(L.lm, true);
    per_mat(L.edge1, true);
    per_mat(L.edges, true);
    per_mat(L.vedge, true);
    L.dv.assign(n, -1);
    for (int a = 0; a < n; ++a)
      if (!top(a)) L.dv[a] = take((int64_t)dup(a) * dup(a) * dup(a) * dup(a));
    // grid problems: X lists (mode order) of the node grid and the hole grid
    L.grid_modes.assign(n, {});
    L.hole_modes.assign(n, {});
    L.grid.assign(n, -1);
    L.hgrid.assign(n, -1);
    for (int a = 0; a < n; ++a) {
      if (top(a)) continue;
      L.grid_modes[a] = sub[a];
      for (int m = 0; m < f; ++m)
        if (leaf_node[m] != a) L.hole_modes[a].push_back(m);
      L.grid[a] = take((int64_t)L.grid_modes[a].size() * dup(a));
      L.hgrid[a] = take((int64_t)L.hole_modes[a].size() * dup(a));
    }
    L.xmat.assign(f, std::vector<int64_t>(n, -1));
    L.xt.assign(f, std::vector<int64_t>(n, -1));
    L.xhole_raw.assign(f, std::vector<int64_t>(n, -1));
    L.xhole.assign(f, std::vector<int64_t>(n, -1));
    for (int m = 0; m < f; ++m) {
      for (int a : path[m]) {
        if (top(a)) continue;
        L.xmat[m][a] = take((int64_t)dup(a) * dup(a));
        L.xt[m][a] = take(nd[a].N);
      }
      for (int a = 0; a < n; ++a) {
        if (top(a) || a == leaf_node[m]) continue;
        L.xhole_raw[m][a] = take((int64_t)dup(a) * dup(a));
        L.xhole[m][a] = take((int64_t)dup(a) * dup(a));
      }
    }
    // constants: noise, leaf grids (and their diagonal matrices), identity
    std::mt19937 gen(23949);
    std::normal_distribution<double> dist;
    for (int a = 0; a < n; ++a) {
      std::vector<double2> z(nd[a].N);
      for (auto& v : z) v = cx(1e-4 * dist(gen));
      P.cdvr_init.push_back({L.noise[a], std::move(z)});
    }
    L.leafx.assign(f, -1);
    leafdiag.assign(f, -1);
    for (int m = 0; m < f; ++m) {
      const int p = (int)D.leaf_x[m].size();
      L.leafx[m] = take(p);
      leafdiag[m] = take((int64_t)p * p);
      std::vector<double2> x(p), dg((size_t)p * p, cx(0.0));
      for (int i = 0; i < p; ++i) {
        x[i] = cx(D.leaf_x[m][i]);
        dg[(size_t)i * p + i] = x[i];
      }
      P.cdvr_init.push_back({L.leafx[m], std::move(x)});
      P.cdvr_init.push_back({leafdiag[m], std::move(dg)});
    }
    {
      const int t = P.tops[0], d = dup(t);
      std::vector<double2> id((size_t)d * d, cx(0.0));
      for (int i = 0; i < d; ++i) id[(size_t)i * d + i] = cx(1.0);
      P.cdvr_init.push_back({L.rho_chi[t], std::move(id)});
    }
    // scratch: eigen tasks, WSD problems, hole chains, corrections
    eig_scr.assign(n, -1);
    for (int a = 0; a < n; ++a)
      if (!top(a)) eig_scr[a] = take((int64_t)8 * dup(a) * dup(a));  // 4 tasks x (U, W)
    wsd_scr.assign(n, {-1, -1});
    for (int a = 0; a < n; ++a) {
      if (top(a)) continue;
      const int64_t dd = (int64_t)dup(a) * dup(a);
      // weighted and plain matrices, weight, transformation, 3 d^2 of products
      if (L.grid_modes[a].size() > 1) wsd_scr[a].first = take((2 * (int64_t)L.grid_modes[a].size() + 5) * dd);
      if (L.hole_modes[a].size() > 1) wsd_scr[a].second = take((2 * (int64_t)L.hole_modes[a].size() + 5) * dd);
    }
    hole_t1.assign(f, std::vector<int64_t>(n, -1));
    hole_t2.assign(f, std::vector<int64_t>(n, -1));
    unw_t.assign(f, std::vector<int64_t>(n, -1));
    for (int m = 0; m < f; ++m)
      for (int a = 0; a < n; ++a) {
        if (L.xhole_raw[m][a] < 0) continue;
        const int p = nd[a].parent;
        hole_t1[m][a] = take(nd[p].N);
        hole_t2[m][a] = take(nd[p].N);
        unw_t[m][a] = take((int64_t)dup(a) * dup(a));
      }
    corr.assign(n, {});
    L.corr_x.assign(n, {});
    L.corr_y.assign(n, {});
    for (int a = 0; a < n; ++a) {
      if (nd[a].bottom()) continue;
      const int dn = dup(a);
      for (size_t k = 0; k < nd[a].children.size(); ++k) {
        const int dc = nd[a].shape[k];
        Corr c;
        const int64_t q = (int64_t)dc * dn * dc * dn;
        if (!top(a)) {
          c.D = take(q);
          c.F = take(q);
          c.E = take(q);
        }
        corr[a].push_back(c);
        L.corr_x[a].push_back(take((int64_t)dc * dc));
        L.corr_y[a].push_back(take((int64_t)dc * dc));
      }
    }
    P.cdvr_size = std::max<int64_t>(cur, kAl);
  }
  std::vector<int64_t> leafdiag, eig_scr;
  std::vector<std::pair<int64_t, int64_t>> wsd_scr;
  std::vector<std::vector<int64_t>> hole_t1, hole_t2, unw_t;
  struct Corr {
    int64_t D = -1, F = -1, E = -1;
  };
  std::vector<std::vector<Corr>> corr;

  // ---- update stages -----------------------------------------------------
  void st_chi() {
    const int64_t t0 = (int64_t)P.gs.size();
    for (int a = 0; a < n; ++a) {
      Plan::SGS g;
      g.in = psi(a);
      g.noise = cd(L.noise[a]);
      g.out = cd(L.chi[a]);
      g.cols = dup(a);
      g.rows = (int)(nd[a].N / g.cols);
      P.gs.push_back(g);
      flops += 16.0 * (double)nd[a].N * g.cols;
    }
    emit(ST_GS, t0, (int64_t)P.gs.size(), t0, (int64_t)P.gs.size(), "cdvr-chi", 0);
  }

  int max_depth() const {
    int m = 0;
    for (auto& g : nd) m = std::max(m, g.depth);
    return m;
  }
  int max_height() const {
    int m = 0;
    for (auto& g : nd) m = std::max(m, g.height);
    return m;
  }

  // rho of Chi, top-down (TreeFunctions::contraction with orthogonal = true)
  void st_rho_chi() {
    for (int dep = 1; dep <= max_depth(); ++dep) {
      TcMark m1 = tc_begin();
      for (int p = 0; p < n; ++p)
        if (nd[p].depth == dep - 1 && !top(p) && !nd[p].bottom())
          tc_mode(cd(L.chi[p]), cd(L.tmpa[p]), cd(L.rho_chi[p]), shape(p), nd[p].last(), 'N', false);
      tc_end(m1, "cdvr-rho-chi");
      TcMark m2 = tc_begin();
      for (int a = 0; a < n; ++a) {
        if (nd[a].depth != dep) continue;
        const int p = nd[a].parent;
        tc_hole(cd(L.rho_chi[a]), cd(L.chi[p]), top(p) ? cd(L.chi[p]) : cd(L.tmpa[p]), shape(p),
                nd[a].child_idx);
      }
      tc_end(m2, "cdvr-rho-chi");
    }
    eigf_stage(2, 1e-8, [&](int a) { return cd(L.rho_chi[a]); }, [&](int a) { return cd(L.isq[a]); },
               0, "cdvr-isqrt-rho-chi");
  }

  // spectral function tasks over the non-top nodes (slot: which scratch pair)
  template <class FA, class FO>
  void eigf_stage(int fn, double eps, FA in, FO out, int slot, const char* name) {
    const int64_t t0 = (int64_t)P.eigf.size();
    for (int a = 0; a < n; ++a) {
      if (top(a)) continue;
      const int64_t dd = (int64_t)dup(a) * dup(a);
      Plan::SEigF e;
      e.A = in(a);
      e.out = out(a);
      e.U = cd(eig_scr[a] + 2 * slot * dd);
      e.W = cd(eig_scr[a] + (2 * slot + 1) * dd);
      e.vals = Ref{-1, 0};
      e.eps = eps;
      e.d = dup(a);
      e.fn = fn;
      P.eigf.push_back(e);
    }
    emit(ST_EIGF, t0, (int64_t)P.eigf.size(), t0, (int64_t)P.eigf.size(), name, 0);
  }

  // X matrices bottom-up along every leaf's path (represent with Xsop)
  void st_xmats() {
    for (int h = 0; h < max_height(); ++h) {
      TcMark m1 = tc_begin();
      for (int m = 0; m < f; ++m) {
        if ((int)path[m].size() <= h) continue;
        const int a = path[m][h];
        if (top(a)) continue;
        if (h == 0) {
          tc_mode(psi(a), cd(L.xt[m][a]), cd(leafdiag[m]), shape(a), 0, 'N', false);
        } else {
          const int c = path[m][h - 1];
          tc_mode(psi(a), cd(L.xt[m][a]), cd(L.xmat[m][c]), shape(a), nd[c].child_idx, 'N', false);
        }
      }
      tc_end(m1, "cdvr-x-represent");
      TcMark m2 = tc_begin();
      for (int m = 0; m < f; ++m) {
        if ((int)path[m].size() <= h) continue;
        const int a = path[m][h];
        if (top(a)) continue;
        tc_hole(cd(L.xmat[m][a]), psi(a), cd(L.xt[m][a]), shape(a), nd[a].last());
      }
      tc_end(m2, "cdvr-x-represent");
    }
  }

  // X holes top-down on Chi with the X matrices of Psi, then unweighted
  void st_xholes() {
    for (int dep = 1; dep <= max_depth(); ++dep) {
      // position 0: the X matrix of the path child (if any, and not the hole node)
      TcMark m1 = tc_begin();
      std::vector<std::vector<Ref>> cur_ref(f, std::vector<Ref>(n));
      for (int m = 0; m < f; ++m)
        for (int a = 0; a < n; ++a) {
          if (nd[a].depth != dep || L.xhole_raw[m][a] < 0) continue;
          const int p = nd[a].parent;
          cur_ref[m][a] = cd(L.chi[p]);
          for (size_t k = 0; k < nd[p].children.size(); ++k) {
            const int c = nd[p].children[k];
            if ((int)k == nd[a].child_idx || !in_sub(c, m)) continue;
            tc_mode(cd(L.chi[p]), cd(hole_t1[m][a]), cd(L.xmat[m][c]), shape(p), (int)k, 'N', false);
            cur_ref[m][a] = cd(hole_t1[m][a]);
          }
        }
      tc_end(m1, "cdvr-x-holes");
      // position 1: the parent's hole on the parent's last index
      TcMark m2 = tc_begin();
      for (int m = 0; m < f; ++m)
        for (int a = 0; a < n; ++a) {
          if (nd[a].depth != dep || L.xhole_raw[m][a] < 0) continue;
          const int p = nd[a].parent;
          if (top(p)) continue;
          tc_mode(cur_ref[m][a], cd(hole_t2[m][a]), cd(L.xhole_raw[m][p]), shape(p), nd[p].last(), 'N',
                  false);
          cur_ref[m][a] = cd(hole_t2[m][a]);
        }
      tc_end(m2, "cdvr-x-holes");
      TcMark m3 = tc_begin();
      for (int m = 0; m < f; ++m)
        for (int a = 0; a < n; ++a) {
          if (nd[a].depth != dep || L.xhole_raw[m][a] < 0) continue;
          const int p = nd[a].parent;
          tc_hole(cd(L.xhole_raw[m][a]), cd(L.chi[p]), cur_ref[m][a], shape(p), nd[a].child_idx);
        }
      tc_end(m3, "cdvr-x-holes");
    }
    TcMark u1 = tc_begin();
    for (int m = 0; m < f; ++m)
      for (int a = 0; a < n; ++a)
        if (L.xhole_raw[m][a] >= 0)
          tc_mm(cd(unw_t[m][a]), cd(L.xhole_raw[m][a]), 'N', cd(L.isq[a]), 'N', dup(a));
    tc_end(u1, "cdvr-x-unweight");
    TcMark u2 = tc_begin();
    for (int m = 0; m < f; ++m)
      for (int a = 0; a < n; ++a)
        if (L.xhole_raw[m][a] >= 0)
          tc_mm(cd(L.xhole[m][a]), cd(L.isq[a]), 'N', cd(unw_t[m][a]), 'N', dup(a));
    tc_end(u2, "cdvr-x-unweight");
  }

  void st_grids() {
    // several matrices: weighted simultaneous diagonalisation
    const int64_t w0 = (int64_t)P.wsd.size();
    for (int a = 0; a < n; ++a) {
      if (top(a)) continue;
      for (int kind = 0; kind < 2; ++kind) {
        const auto& modes = kind == 0 ? L.grid_modes[a] : L.hole_modes[a];
        if (modes.size() < 2) continue;
        Plan::SWSD w;
        w.W = mat(P.rho_off[a]);
        w.trafo = cd(kind == 0 ? L.trafo[a] : L.htrafo[a]);
        w.grid = cd(kind == 0 ? L.grid[a] : L.hgrid[a]);
        w.scratch = cd(kind == 0 ? wsd_scr[a].first : wsd_scr[a].second);
        w.d = dup(a);
        w.n = (int)modes.size();
        w.first = (int)P.wsd_terms.size();
        for (int m : modes) P.wsd_terms.push_back(cd(kind == 0 ? L.xmat[m][a] : L.xhole[m][a]));
        P.wsd.push_back(w);
        P.wsd_max_n = std::max(P.wsd_max_n, w.n);
        P.wsd_max_d = std::max(P.wsd_max_d, w.d);
      }
    }
    emit(ST_WSD, w0, (int64_t)P.wsd.size(), w0, (int64_t)P.wsd.size(), "cdvr-grids-wsd", 0);
    // one matrix: eigenvectors
    const int64_t e0 = (int64_t)P.eigf.size();
    for (int a = 0; a < n; ++a) {
      if (top(a)) continue;
      const int64_t dd = (int64_t)dup(a) * dup(a);
      for (int kind = 0; kind < 2; ++kind) {
        const auto& modes = kind == 0 ? L.grid_modes[a] : L.hole_modes[a];
        if (modes.size() != 1) continue;
        Plan::SEigF e;
        e.A = cd(kind == 0 ? L.xmat[modes[0]][a] : L.xhole[modes[0]][a]);
        e.out = cd(kind == 0 ? L.trafo[a] : L.htrafo[a]);
        e.U = cd(eig_scr[a] + (2 + 2 * kind) * dd);
        e.W = cd(eig_scr[a] + (3 + 2 * kind) * dd);
        e.vals = cd(kind == 0 ? L.grid[a] : L.hgrid[a]);
        e.eps = 0;
        e.d = dup(a);
        e.fn = 4;
        P.eigf.push_back(e);
      }
    }
    emit(ST_EIGF, e0, (int64_t)P.eigf.size(), e0, (int64_t)P.eigf.size(), "cdvr-grids-eig", 0);
  }

  // MatrixTensorTree, GridTransformation, bottom-up / top-down coefficients
  void st_edges() {
    eigf_stage(1, 0.0, [&](int a) { return mat(P.rho_off[a]); }, [&](int a) { return cd(L.sqrt_rho[a]); },
               0, "cdvr-sqrt-rho");
    eigf_stage(2, 1e-7, [&](int a) { return mat(P.rho_off[a]); }, [&](int a) { return cd(L.binv[a]); }, 1,
               "cdvr-edges");
    eigf_stage(3, 1e-6, [&](int a) { return mat(P.rho_off[a]); }, [&](int a) { return cd(L.sqrho[a]); },
               2, "cdvr-sqrt-rho-reg");
    TcMark m1 = tc_begin();
    for (int a = 0; a < n; ++a) {
      if (top(a)) continue;
      const int d = dup(a);
      tc_mm(cd(L.g[a]), cd(L.htrafo[a]), 'N', cd(L.sqrt_rho[a]), 'N', d);
      tc_mm(cd(L.lm[a]), cd(L.htrafo[a]), 'N', cd(L.sqrho[a]), 'N', d);
      tc_mm(cd(L.edge1[a]), cd(L.trafo[a]), 'C', cd(L.binv[a]), 'N', d);
    }
    tc_end(m1, "cdvr-edges");
    TcMark m2 = tc_begin();
    for (int a = 0; a < n; ++a)
      if (!top(a)) tc_mm(cd(L.edges[a]), cd(L.edge1[a]), 'N', cd(L.htrafo[a]), 'H', dup(a));
    tc_end(m2, "cdvr-edges");
    // node tensors on the grids: children's trafo, then G = htrafo sqrt(rho) on the last index
    chain(
        [&](int a, std::vector<std::pair<Ref, std::pair<int, char>>>& ops) {
          if (!nd[a].bottom())
            for (size_t k = 0; k < nd[a].children.size(); ++k)
              ops.push_back({cd(L.trafo[nd[a].children[k]]), {(int)k, 'N'}});
          if (!top(a)) ops.push_back({cd(L.g[a]), {nd[a].last(), 'N'}});
        },
        [&](int a) { return psi(a); }, [&](int a) { return cd(L.at[a]); }, false, "cdvr-grid-nodes");
    TcMark m3 = tc_begin();
    for (int a = 0; a < n; ++a) {
      if (top(a)) continue;
      tc_mode(cd(L.at[a]), cd(L.cup[a]), cd(L.edges[a]), shape(a), nd[a].last(), 'N', false);
      const int p = nd[a].parent;
      tc_mode(cd(L.at[p]), cd(L.cdown[a]), cd(L.edges[a]), shape(p), nd[a].child_idx, 'T', false);
    }
    tc_end(m3, "cdvr-coefficients");
  }

  // per node a chain of mode products (in -> ... -> out); with `add` the
  // last product adds into out.  Ping-pong through tmpa / tmpb.
  template <class FOps, class FIn, class FOut>
  void chain(FOps ops_of, FIn in_of, FOut out_of, bool add, const char* name) {
    std::vector<std::vector<std::pair<Ref, std::pair<int, char>>>> ops(n);
    size_t maxlen = 0;
    for (int a = 0; a < n; ++a) {
      ops_of(a, ops[a]);
      maxlen = std::max(maxlen, ops[a].size());
    }
    for (size_t pos = 0; pos < maxlen; ++pos) {
      TcMark m = tc_begin();
      for (int a = 0; a < n; ++a) {
        const size_t len = ops[a].size();
        if (pos >= len) continue;
        const Ref in = pos == 0 ? in_of(a) : cd(pos % 2 == 1 ? L.tmpa[a] : L.tmpb[a]);
        const bool last = pos + 1 == len;
        const Ref out = last ? out_of(a) : cd(pos % 2 == 0 ? L.tmpa[a] : L.tmpb[a]);
        const auto& o = ops[a][pos];
        tc_mode(in, out, o.first, shape(a), o.second.first, o.second.second, last && add);
      }
      tc_end(m, name);
    }
  }

  // node and edge potentials (UpdateNodeDVR / UpdateEdgeDVR, fillX*)
  Ref hole_grid_of(int a, int m) const {
    // the hole grid tree of mode m at node a receives, in the reference,
    // the diagonal of the X matrix with the same rank among the active grids
    const auto& xs = L.hole_modes[a];
    int j = -1;
    if (D.aligned) {
      j = (int)(std::find(xs.begin(), xs.end(), m) - xs.begin());
    } else {
      j = 0;
      for (int l = 0; l < m; ++l)
        if (!in_sub(a, l)) ++j;
    }
    return cd(L.hgrid[a] + (int64_t)j * dup(a));
  }
  Ref node_grid_of(int c, int m) const {
    const auto& xs = L.grid_modes[c];
    const int j = (int)(std::find(xs.begin(), xs.end(), m) - xs.begin());
    return cd(L.grid[c] + (int64_t)j * dup(c));
  }
  void vpot_task(Ref out, const std::vector<int>& dims, const std::vector<Plan::SVCoord>& coords) {
    Plan::SVPot v;
    v.out = out;
    v.order = (int)dims.size();
    int64_t tot = 1;
    for (int i = 0; i < 6; ++i) v.dims[i] = i < v.order ? dims[i] : 1;
    for (int x : dims) tot *= x;
    v.n = tot;
    v.first = (int)P.vcoords.size();
    for (auto& c : coords) P.vcoords.push_back(c);
    const int task = (int)P.vpot.size();
    P.vpot.push_back(v);
    for (int64_t s = 0; s < tot; s += 256) P.vpot_tiles.push_back(make_int2(task, (int)s));
  }
  void st_potential() {
    const int64_t t0 = (int64_t)P.vpot.size(), tile0 = (int64_t)P.vpot_tiles.size();
    for (int a = 0; a < n; ++a) {
      std::vector<Plan::SVCoord> co(f);
      if (nd[a].bottom()) {
        const int m = nd[a].leaf_mode;
        co[m] = Plan::SVCoord{cd(L.leafx[m]), 0};
      } else {
        for (size_t k = 0; k < nd[a].children.size(); ++k) {
          const int c = nd[a].children[k];
          for (int m : sub[c]) co[m] = Plan::SVCoord{node_grid_of(c, m), (int)k};
        }
      }
      if (!top(a))
        for (int m = 0; m < f; ++m)
          if (!in_sub(a, m)) co[m] = Plan::SVCoord{hole_grid_of(a, m), nd[a].last()};
      vpot_task(cd(L.vnode[a]), shape(a), co);
    }
    for (int a = 0; a < n; ++a) {
      if (top(a)) continue;
      std::vector<Plan::SVCoord> co(f);
      for (int m = 0; m < f; ++m)
        co[m] = in_sub(a, m) ? Plan::SVCoord{node_grid_of(a, m), 0} : Plan::SVCoord{hole_grid_of(a, m), 1};
      vpot_task(cd(L.vedge[a]), {dup(a), dup(a)}, co);
    }
    emit(ST_VPOT, t0, (int64_t)P.vpot.size(), tile0, (int64_t)P.vpot_tiles.size(), "cdvr-potential", 0);
  }

  void st_delta_v() {
    for (int h = 0; h <= max_height(); ++h) {
      const int64_t t0 = (int64_t)P.dvl.size(), tile0 = (int64_t)P.dvl_tiles.size();
      for (int a = 0; a < n; ++a) {
        if (nd[a].height != h || top(a)) continue;
        Plan::SDVL t;
        t.cup = cd(L.cup[a]);
        t.vnode = cd(L.vnode[a]);
        t.vedge = cd(L.vedge[a]);
        t.dv = cd(L.dv[a]);
        t.d = dup(a);
        t.bef = (int)(nd[a].N / t.d);
        const int task = (int)P.dvl.size();
        P.dvl.push_back(t);
        const int64_t tot = (int64_t)t.d * t.d * t.d * t.d;
        for (int64_t s = 0; s < tot; s += 256) P.dvl_tiles.push_back(make_int2(task, (int)s));
        flops += 8.0 * (double)t.d * t.d * t.d * t.bef;
      }
      emit(ST_DVL, t0, (int64_t)P.dvl.size(), tile0, (int64_t)P.dvl_tiles.size(), "cdvr-dv-local", 0);
      if (h == 0) continue;
      // D and F (doubleHoleContraction), then E = dv_child D', then dv += F' E per child index
      TcMark m1 = tc_begin();
      int maxk = 0;
      for (int a = 0; a < n; ++a) {
        if (nd[a].height != h || top(a)) continue;
        const int nk = (int)nd[a].children.size();
        maxk = std::max(maxk, nk);
        for (int k = 0; k < nk; ++k) {
          const int c = nd[a].children[k];
          dhole(cd(corr[a][k].D), cd(L.cdown[c]), cd(L.cup[a]), a, k);
          dhole(cd(corr[a][k].F), cd(L.cup[a]), cd(L.cdown[c]), a, k);
        }
      }
      tc_end(m1, "cdvr-dv-holes");
      TcMark m2 = tc_begin();
      for (int a = 0; a < n; ++a) {
        if (nd[a].height != h || top(a)) continue;
        for (size_t k = 0; k < nd[a].children.size(); ++k) build_e(a, (int)k);
      }
      tc_end(m2, "cdvr-dv-e");
      for (int k = 0; k < maxk; ++k) {
        TcMark m3 = tc_begin();
        for (int a = 0; a < n; ++a) {
          if (nd[a].height != h || top(a) || k >= (int)nd[a].children.size()) continue;
          contract_ef(a, k);
        }
        tc_end(m3, "cdvr-dv-ef");
      }
    }
  }
  // C[a, b, c, e] = sum over all indices but (k, last) of conj(A[..a@k..b@last]) B[..c@k..e@last]
  void dhole(Ref C, Ref A, Ref B, int a, int k) {
    const auto& s = nd[a].shape;
    const int last = nd[a].last();
    int64_t befk = 1, mid = 1;
    for (int i = 0; i < k; ++i) befk *= s[i];
    for (int i = k + 1; i < last; ++i) mid *= s[i];
    const int dk = s[k], dn = s[last];
    Plan::STC t = tc0();
    t.A = A;
    t.B = B;
    t.C = C;
    t.M0 = dk;
    t.am0 = befk;
    t.M1 = dn;
    t.am1 = befk * dk * mid;
    t.K0 = (int)befk;
    t.ak0 = 1;
    t.K1 = (int)mid;
    t.ak1 = befk * dk;
    t.conjA = 1;
    t.N0 = dk;
    t.bn0 = befk;
    t.N1 = dn;
    t.bn1 = befk * dk * mid;
    t.bk0 = 1;
    t.bk1 = befk * dk;
    t.cm0 = 1;
    t.cm1 = dk;
    t.cn0 = (int64_t)dk * dn;
    t.cn1 = (int64_t)dk * dn * dk;
    tc_push(t);
  }
  // buildE: E[i0, i1, i2, i3] = sum_{l1, l2} dv_c[i0, i1, l1, l2] D[l2, i3, l1, i2]
  void build_e(int a, int k) {
    const int c = nd[a].children[k];
    const int64_t dc = nd[a].shape[k], dn = dup(a);
    Plan::STC t = tc0();
    t.A = cd(L.dv[c]);
    t.B = cd(corr[a][k].D);
    t.C = cd(corr[a][k].E);
    t.M0 = t.M1 = (int)dc;
    t.am0 = 1;
    t.am1 = dc;
    t.K0 = t.K1 = (int)dc;
    t.ak0 = dc * dc;
    t.ak1 = dc * dc * dc;
    t.bk0 = dc * dn;
    t.bk1 = 1;
    t.N0 = t.N1 = (int)dn;
    t.bn0 = dc * dn * dc;
    t.bn1 = dc;
    t.cm0 = 1;
    t.cm1 = dc;
    t.cn0 = dc * dc;
    t.cn1 = dc * dc * dn;
    tc_push(t);
  }
  // contractEF: dv[i0, i1, i2, i3] += sum_{l1, l2} F[l1, i0, l2, i1] E[l1, l2, i2, i3]
  void contract_ef(int a, int k) {
    const int64_t dc = nd[a].shape[k], dn = dup(a);
    Plan::STC t = tc0();
    t.A = cd(corr[a][k].F);
    t.B = cd(corr[a][k].E);
    t.C = cd(L.dv[a]);
    t.M0 = t.M1 = (int)dn;
    t.am0 = dc;
    t.am1 = dc * dn * dc;
    t.K0 = t.K1 = (int)dc;
    t.ak0 = 1;
    t.ak1 = dc * dn;
    t.bk0 = 1;
    t.bk1 = dc;
    t.N0 = t.N1 = (int)dn;
    t.bn0 = dc * dc;
    t.bn1 = dc * dc * dn;
    t.cm0 = 1;
    t.cm1 = dn;
    t.cn0 = dn * dn;
    t.cn1 = dn * dn * dn;
    t.add = 1;
    tc_push(t);
  }

  // ---- apply stages ------------------------------------------------------
  void st_apply() {
    // Xi = (children's trafo) (htrafo sqrt(rho) regularised on the last index) Phi
    chain(
        [&](int a, std::vector<std::pair<Ref, std::pair<int, char>>>& ops) {
          if (!nd[a].bottom())
            for (size_t k = 0; k < nd[a].children.size(); ++k)
              ops.push_back({cd(L.trafo[nd[a].children[k]]), {(int)k, 'N'}});
          if (!top(a)) ops.push_back({cd(L.lm[a]), {nd[a].last(), 'N'}});
        },
        [&](int a) { return psi(a); }, [&](int a) { return cd(L.xi[a]); }, false, "cdvr-apply-in");
    {  // V Xi
      const int64_t t0 = (int64_t)P.ew.size(), tile0 = (int64_t)P.ew_tiles.size();
      for (int a = 0; a < n; ++a) {
        Plan::SEW e;
        e.v = cd(L.vnode[a]);
        e.in = cd(L.xi[a]);
        e.out = cd(L.vx[a]);
        e.n = nd[a].N;
        e.add = 0;
        const int task = (int)P.ew.size();
        P.ew.push_back(e);
        for (int64_t s = 0; s < e.n; s += 1024) P.ew_tiles.push_back(make_int2(task, (int)s));
        flops += 6.0 * (double)e.n;
      }
      emit(ST_EW, t0, (int64_t)P.ew.size(), tile0, (int64_t)P.ew_tiles.size(), "cdvr-apply-v", 0);
    }
    // corrections of the children's edges (applyCorrection)
    int maxk = 0;
    TcMark m1 = tc_begin();
    for (int a = 0; a < n; ++a) {
      if (nd[a].bottom()) continue;
      maxk = std::max(maxk, (int)nd[a].children.size());
      for (size_t k = 0; k < nd[a].children.size(); ++k)
        tc_hole(cd(L.corr_x[a][k]), cd(L.cdown[nd[a].children[k]]), cd(L.xi[a]), shape(a), (int)k);
    }
    tc_end(m1, "cdvr-apply-x");
    TcMark m2 = tc_begin();
    for (int a = 0; a < n; ++a) {
      if (nd[a].bottom()) continue;
      for (size_t k = 0; k < nd[a].children.size(); ++k) {
        // y(l0, l1) = sum_{l2, l3} dv(l0, l1, l2, l3) x(l3, l2)
        const int c = nd[a].children[k];
        const int64_t dc = nd[a].shape[k];
        Plan::STC t = tc0();
        t.A = cd(L.dv[c]);
        t.B = cd(L.corr_x[a][k]);
        t.C = cd(L.corr_y[a][k]);
        t.M0 = t.M1 = (int)dc;
        t.am0 = 1;
        t.am1 = dc;
        t.K0 = t.K1 = (int)dc;
        t.ak0 = dc * dc;
        t.ak1 = dc * dc * dc;
        t.bk0 = dc;
        t.bk1 = 1;
        t.cm0 = 1;
        t.cm1 = dc;
        tc_push(t);
      }
    }
    tc_end(m2, "cdvr-apply-dv");
    for (int k = 0; k < maxk; ++k) {
      TcMark m3 = tc_begin();
      for (int a = 0; a < n; ++a) {
        if (nd[a].bottom() || k >= (int)nd[a].children.size()) continue;
        tc_mode(cd(L.cdown[nd[a].children[k]]), cd(L.vx[a]), cd(L.corr_y[a][k]), shape(a), k, 'N', true);
      }
      tc_end(m3, "cdvr-apply-corr");
    }
    // back: children's trafo^dagger, (htrafo sqrt(rho))^dagger, added to H Phi
    chain(
        [&](int a, std::vector<std::pair<Ref, std::pair<int, char>>>& ops) {
          if (!nd[a].bottom())
            for (size_t k = 0; k < nd[a].children.size(); ++k)
              ops.push_back({cd(L.trafo[nd[a].children[k]]), {(int)k, 'H'}});
          if (!top(a)) ops.push_back({cd(L.lm[a]), {nd[a].last(), 'H'}});
        },
        [&](int a) { return cd(L.vx[a]); }, [&](int a) { return hphi(a); }, true, "cdvr-apply-out");
  }
};

}  // namespace

double cdvr_plan(Plan& P, const CdvrDesc& D, int part) {
  CdvrBuilder b(P, D);
  return part == 0 ? b.update() : b.apply();
}

}  // namespace qt
