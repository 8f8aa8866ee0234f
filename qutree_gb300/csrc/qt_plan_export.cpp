// qt_plan_export.cpp -- host-only view of the sweep plan (no CUDA calls).
//
// Builds the same plan qt_prepare builds and hands its symbolic task tables
// (buffer id + element offset instead of device pointers) to the caller.
// The CPU test suite interprets these tables with numpy to check the
// planner's schedule on machines without a GPU.  Compiled with g++ into
// libqtplan.so, separate from the CUDA library.
#include <cstring>
#include <string>
#include <vector>

#include "qt_internal.h"

namespace {
struct Handle {
  qt::Plan plan;
};

void put_ref(std::vector<int64_t>& v, const qt::Ref& r) {
  v.push_back(r.buf);
  v.push_back(r.off);
}
}  // namespace

extern "C" {

static void* build_handle(int n_nodes, const int* order, const int* dims, const int* parent, const int* child_idx,
                          const int* leaf_mode, int n_ops, const int* op_kind, const int* op_dim,
                          const int64_t* op_off, const double* op_data, int n_terms, const double* coeff,
                          const int* term_ptr, const int* term_mode, const int* term_op, int flavour,
                          int prec, int64_t budget, char* err, int errlen, const qt::CdvrDesc* cd) {
  const bool grad = (flavour & 0x1000) != 0;
  flavour &= ~0x1000;
  std::vector<qt::NodeGeo> nodes(n_nodes);
  int p = 0;
  for (int i = 0; i < n_nodes; ++i) {
    for (int k = 0; k < order[i]; ++k) nodes[i].shape.push_back(dims[p + k]);
    p += order[i];
    nodes[i].parent = parent[i];
    nodes[i].child_idx = child_idx[i];
    nodes[i].leaf_mode = leaf_mode[i];
  }
  // same operator repacking as qt_sop_upload
  qt::OpTable ops;
  int64_t cur = 0;
  for (int i = 0; i < n_ops; ++i) {
    int64_t n = op_kind[i] == 0 ? (int64_t)op_dim[i] * op_dim[i] : op_dim[i];
    ops.kind.push_back(op_kind[i]);
    ops.dim.push_back(op_dim[i]);
    ops.off.push_back(cur);
    ops.data.resize(2 * (cur + n), 0.0);
    std::memcpy(ops.data.data() + 2 * cur, op_data + 2 * op_off[i], sizeof(double) * 2 * n);
    cur = (cur + n + 15) / 16 * 16;
  }
  ops.data.resize(2 * (cur > 16 ? cur : 16), 0.0);
  qt::SopDesc s;
  s.n_terms = n_terms;
  for (int l = 0; l < n_terms; ++l) s.coeff.push_back(make_double2(coeff[2 * l], coeff[2 * l + 1]));
  s.ptr.assign(term_ptr, term_ptr + n_terms + 1);
  s.mode.assign(term_mode, term_mode + s.ptr[n_terms]);
  s.op.assign(term_op, term_op + s.ptr[n_terms]);
  Handle* h = new Handle();
  std::string msg = qt::build_plan(h->plan, nodes, ops, s, flavour, prec, budget, grad, cd);
  if (!msg.empty()) {
    if (err && errlen > 0) {
      std::strncpy(err, msg.c_str(), errlen - 1);
      err[errlen - 1] = 0;
    }
    delete h;
    return nullptr;
  }
  h->plan.ops_size = (int64_t)ops.data.size() / 2;
  return h;
}

void* qtp_build(int n_nodes, const int* order, const int* dims, const int* parent, const int* child_idx,
                const int* leaf_mode, int n_ops, const int* op_kind, const int* op_dim,
                const int64_t* op_off, const double* op_data, int n_terms, const double* coeff,
                const int* term_ptr, const int* term_mode, const int* term_op, int flavour,
                int prec, int64_t budget, char* err, int errlen) {
  return build_handle(n_nodes, order, dims, parent, child_idx, leaf_mode, n_ops, op_kind, op_dim, op_off,
                      op_data, n_terms, coeff, term_ptr, term_mode, term_op, flavour, prec, budget, err,
                      errlen, nullptr);
}

// the same with a CDVR potential (arguments of qt_cdvr_upload appended)
void* qtp_build_cdvr(int n_nodes, const int* order, const int* dims, const int* parent, const int* child_idx,
                     const int* leaf_mode, int n_ops, const int* op_kind, const int* op_dim,
                     const int64_t* op_off, const double* op_data, int n_terms, const double* coeff,
                     const int* term_ptr, const int* term_mode, const int* term_op, int flavour, int prec,
                     int64_t budget, char* err, int errlen, int n_modes, const int* leaf_dim,
                     const double* leaf_x, int n_pterms, const double* pcoeff, const int* pptr,
                     const int* pmode, const int* ppow, int flags) {
  qt::CdvrDesc d;
  int64_t off = 0;
  for (int m = 0; m < n_modes; ++m) {
    d.leaf_x.emplace_back(leaf_x + off, leaf_x + off + leaf_dim[m]);
    off += leaf_dim[m];
  }
  d.coeff.assign(pcoeff, pcoeff + n_pterms);
  d.ptr.assign(pptr, pptr + n_pterms + 1);
  d.mode.assign(pmode, pmode + pptr[n_pterms]);
  d.power.assign(ppow, ppow + pptr[n_pterms]);
  d.aligned = (flags & 1) != 0;
  return build_handle(n_nodes, order, dims, parent, child_idx, leaf_mode, n_ops, op_kind, op_dim, op_off,
                      op_data, n_terms, coeff, term_ptr, term_mode, term_op, flavour, prec, budget, err,
                      errlen, &d);
}

void qtp_free(void* h) { delete (Handle*)h; }

// Table ids: 0 stages, 1 mp, 2 hp, 3 acc, 4 acc_terms, 5 lin, 6 lin_terms,
// 7 eig, 8 proj, 9 sizes, 10 identities, 11 rho_off, 12 rhoinv_off,
// 13 hslot, 14 cslot, 18 cvt, 15 mp alphas, 16 lin coeffs, 17 stats (doubles),
// 40-43 tensor-core mode-product tiles, stage ranges, tasks and classic tiles,
// 44-48 hole-product splits, tiles, launches, stage launch ranges, workspace,
// 49-51 accumulation, small matrix-product and conversion tiles.
// qtp_size returns the element count, qtp_get copies.
static void table(const qt::Plan& P, int what, std::vector<int64_t>& v, std::vector<double>& dv) {
  v.clear();
  dv.clear();
  switch (what) {
    case 0:
      for (auto& s : P.stages) {
        v.push_back(s.kind);
        v.push_back(s.first_task);
        v.push_back(s.n_tasks);
        v.push_back(s.first_tile);
        v.push_back(s.n_tiles);
      }
      break;
    case 1:
      for (auto& t : P.mp) {
        put_ref(v, t.in);
        put_ref(v, t.out);
        put_ref(v, t.h);
        v.push_back(t.before);
        v.push_back(t.a_in);
        v.push_back(t.a_out);
        v.push_back(t.after);
        v.push_back(t.diag);
      }
      break;
    case 2:
      for (auto& t : P.hp) {
        put_ref(v, t.A);
        put_ref(v, t.B);
        put_ref(v, t.S);
        v.push_back(t.before);
        v.push_back(t.a);
        v.push_back(t.after);
      }
      break;
    case 3:
      for (auto& t : P.acc) {
        put_ref(v, t.out);
        v.push_back(t.alpha_ref.buf >= 0 ? 2 : (t.alpha_param ? 1 : 0));
        v.push_back(t.alpha_ref.off);
        v.push_back(t.rows);
        v.push_back(t.d);
        v.push_back(t.first);
        v.push_back(t.count);
        v.push_back(t.add);
      }
      break;
    case 4:
      for (auto& t : P.acc_terms) {
        put_ref(v, t.H);
        put_ref(v, t.X);
      }
      break;
    case 5:
      for (auto& t : P.lin) {
        put_ref(v, t.out);
        v.push_back(t.d);
        v.push_back(t.first);
        v.push_back(t.count);
      }
      break;
    case 6:
      for (auto& t : P.lin_terms) put_ref(v, t.M);
      break;
    case 7:
      for (auto& t : P.eig) {
        put_ref(v, t.rho);
        put_ref(v, t.rhoinv);
        put_ref(v, t.U);
        v.push_back(t.d);
      }
      break;
    case 8:
      for (auto& t : P.proj) {
        put_ref(v, t.S);
        put_ref(v, t.D);
        put_ref(v, t.rhoinv);
        put_ref(v, t.Sinv);
        put_ref(v, t.P);
        put_ref(v, t.M2);
        v.push_back(t.d);
      }
      break;
    case 9:
      v = {P.psi_arena, P.mats_size, P.scratch_size, P.ops_size, P.energy_off[0], P.stop_off[0], P.prec,
           P.keep_size, P.main_end, (int64_t)P.tops.size()};
      for (size_t k = 0; k < P.tops.size(); ++k) {
        v.push_back(P.tops[k]);
        v.push_back(P.energy_off[k]);
        v.push_back(P.stop_off[k]);
      }
      break;
    case 20:  // SCF segments per node: up, down, apply stage ranges
      for (size_t a = 0; a < P.scf_up_b.size(); ++a) {
        v.push_back(P.scf_up_b[a]);
        v.push_back(P.scf_up_e[a]);
        v.push_back(P.scf_down_b[a]);
        v.push_back(P.scf_down_e[a]);
        v.push_back(P.scf_apply_b[a]);
        v.push_back(P.scf_apply_e[a]);
      }
      break;
    case 21:
      v = {P.kry_in, P.kry_out, P.kry_size, P.scf ? 1 : 0};
      break;
    case 22:  // matrix-product tasks: out ref, d, first, count, trans_b
      for (auto& t : P.mm) {
        put_ref(v, t.out);
        v.push_back(t.d);
        v.push_back(t.first);
        v.push_back(t.count);
        v.push_back(t.trans_b);
      }
      break;
    case 23:
      for (auto& t : P.mm_terms) {
        put_ref(v, t.A);
        put_ref(v, t.B);
      }
      break;
    case 19:
      for (auto& t : P.grad) {
        put_ref(v, t.eout);
        put_ref(v, t.rho);
        put_ref(v, t.m3);
        put_ref(v, t.h00);
        put_ref(v, t.s00);
        put_ref(v, t.alpha);
        v.push_back(t.d);
        v.push_back(t.write_alpha);
      }
      break;
    case 18:
      for (auto& t : P.cvt) {
        put_ref(v, t.src);
        put_ref(v, t.dst);
        v.push_back(t.n);
        v.push_back(t.dir);
      }
      break;
    case 10:
      for (auto& id : P.identities) {
        v.push_back(id.first);
        v.push_back(id.second);
      }
      break;
    case 11:
      v = P.rho64_off;
      break;
    case 12:
      v = P.rhoinv64_off;
      break;
    case 13:  // (term, node, hslot, cslot) of every active pair
      for (size_t l = 0; l < P.term_nodes.size(); ++l)
        for (size_t i = 0; i < P.term_nodes[l].size(); ++i) {
          v.push_back((int64_t)l);
          v.push_back(P.term_nodes[l][i]);
          v.push_back(P.term_hslot[l][i]);
          v.push_back(P.term_cslot[l][i]);
        }
      break;
    case 15:
      for (auto& t : P.mp) {
        dv.push_back(t.alpha.x);
        dv.push_back(t.alpha.y);
      }
      break;
    case 16:
      for (auto& t : P.lin_terms) {
        dv.push_back(t.c.x);
        dv.push_back(t.c.y);
      }
      break;
    case 17:
      dv = {P.stats.ref_flops, P.stats.exec_flops, (double)P.main_end,
            (double)P.stats.rep_chains, (double)P.stats.mf_chains, (double)P.stats.app_chains};
      break;
    // ---- CDVR ----
    case 24:
      for (auto& t : P.tc) {
        put_ref(v, t.A);
        put_ref(v, t.B);
        put_ref(v, t.C);
        for (int64_t x : {(int64_t)t.M0, (int64_t)t.M1, (int64_t)t.N0, (int64_t)t.N1, (int64_t)t.K0,
                          (int64_t)t.K1, (int64_t)t.conjA, (int64_t)t.conjB, (int64_t)t.add, t.am0, t.am1,
                          t.ak0, t.ak1, t.bk0, t.bk1, t.bn0, t.bn1, t.cm0, t.cm1, t.cn0, t.cn1})
          v.push_back(x);
      }
      break;
    case 25:
      for (auto& t : P.gs) {
        put_ref(v, t.in);
        put_ref(v, t.noise);
        put_ref(v, t.out);
        v.push_back(t.rows);
        v.push_back(t.cols);
      }
      break;
    case 26:
      for (auto& t : P.eigf) {
        put_ref(v, t.A);
        put_ref(v, t.out);
        put_ref(v, t.U);
        put_ref(v, t.W);
        put_ref(v, t.vals);
        v.push_back(t.d);
        v.push_back(t.fn);
      }
      break;
    case 27:
      for (auto& t : P.wsd) {
        put_ref(v, t.W);
        put_ref(v, t.trafo);
        put_ref(v, t.grid);
        put_ref(v, t.scratch);
        v.push_back(t.d);
        v.push_back(t.n);
        v.push_back(t.first);
      }
      break;
    case 28:
      for (auto& r : P.wsd_terms) put_ref(v, r);
      break;
    case 29:
      for (auto& t : P.vpot) {
        put_ref(v, t.out);
        v.push_back(t.n);
        v.push_back(t.order);
        v.push_back(t.first);
        for (int i = 0; i < 6; ++i) v.push_back(t.dims[i]);
      }
      break;
    case 30:
      for (auto& t : P.tc) {
        dv.push_back(t.alpha.x);
        dv.push_back(t.alpha.y);
      }
      break;
    case 31:
      for (auto& t : P.eigf) dv.push_back(t.eps);
      break;
    case 32:
      for (auto& init : P.cdvr_init)
        for (auto& x : init.second) {
          dv.push_back(x.x);
          dv.push_back(x.y);
        }
      break;
    case 33:
      for (auto& c : P.vcoords) {
        put_ref(v, c.grid);
        v.push_back(c.index);
      }
      break;
    case 34:
      for (auto& t : P.dvl) {
        put_ref(v, t.cup);
        put_ref(v, t.vnode);
        put_ref(v, t.vedge);
        put_ref(v, t.dv);
        v.push_back(t.bef);
        v.push_back(t.d);
      }
      break;
    case 35:
      for (auto& t : P.ew) {
        put_ref(v, t.v);
        put_ref(v, t.in);
        put_ref(v, t.out);
        v.push_back(t.n);
        v.push_back(t.add);
      }
      break;
    case 36:
      for (auto& init : P.cdvr_init) {
        v.push_back(init.first);
        v.push_back((int64_t)init.second.size());
      }
      break;
    case 37:
      v = {P.cdvr ? 1 : 0, P.cdvr_size, P.cdvr_update_begin, P.cdvr_update_end, P.apply_begin};
      break;
    case 38:  // per node: CDVR offsets
      if (P.cdvr)
        for (size_t a = 0; a < P.nodes.size(); ++a) {
          const auto& L = P.cd;
          v.push_back(L.trafo[a]);
          v.push_back(L.htrafo[a]);
          v.push_back(L.grid[a]);
          v.push_back(L.hgrid[a]);
          v.push_back((int64_t)L.grid_modes[a].size());
          v.push_back((int64_t)L.hole_modes[a].size());
          v.push_back(L.vnode[a]);
          v.push_back(L.vedge[a]);
          v.push_back(L.dv[a]);
          v.push_back(L.cup[a]);
          v.push_back(L.cdown[a]);
          v.push_back(L.at[a]);
          v.push_back(L.xi[a]);
          v.push_back(L.vx[a]);
        }
      break;
    case 39:  // (mode, node, X matrix, raw hole, unweighted hole)
      if (P.cdvr)
        for (size_t m = 0; m < P.cd.xmat.size(); ++m)
          for (size_t a = 0; a < P.nodes.size(); ++a) {
            v.push_back((int64_t)m);
            v.push_back((int64_t)a);
            v.push_back(P.cd.xmat[m][a]);
            v.push_back(P.cd.xhole_raw[m][a]);
            v.push_back(P.cd.xhole[m][a]);
          }
      break;
    case 40:  // tensor-core mode-product tiles: (task, tile of kMpOzSub x kMpOzRows rows)
      for (auto& t : P.mp_oz_tiles) {
        v.push_back(t.x);
        v.push_back(t.y);
      }
      break;
    case 41:  // per stage: its tensor-core tiles and tasks (first, count, first, count)
      for (auto& st : P.stages) {
        v.push_back(st.oz0);
        v.push_back(st.noz);
        v.push_back(st.ozt0);
        v.push_back(st.nozt);
      }
      break;
    case 42:  // tensor-core tasks: (task, byte offset of its digits of h in B_OZ)
      for (int t : P.mp_oz_tasks) {
        v.push_back(t);
        v.push_back(P.mp[t].oz_h);
      }
      break;
    case 43:  // classic mode-product tiles: (task, first slot)
      for (auto& t : P.mp_tiles) {
        v.push_back(t.x);
        v.push_back(t.y);
      }
      break;
    case 44:  // hole-product tasks: (splits, kchunk, workspace offset, register tile rows, cols)
      for (auto& t : P.hp) {
        v.push_back(t.splits);
        v.push_back(t.kchunk);
        v.push_back(t.ws);
        v.push_back(t.rows);
        v.push_back(t.cols);
      }
      break;
    case 45:  // hole-product tiles: (task, output tile, reduction range)
      for (auto& t : P.hp_tiles) {
        v.push_back(t.x);
        v.push_back(t.y);
        v.push_back(t.z);
      }
      break;
    case 46:  // hole-product launches: (rows, cols, first tile, tile count)
      for (auto& t : P.hp_segs) {
        v.push_back(t.x);
        v.push_back(t.y);
        v.push_back(t.z);
        v.push_back(t.w);
      }
      break;
    case 47:  // per stage: first launch, launches, partial tiles summed (0/1)
      for (auto& st : P.stages) {
        v.push_back(st.seg0);
        v.push_back(st.nseg);
        v.push_back(st.aux);
      }
      break;
    case 48:  // hole-product workspace size (elements)
      v.push_back(P.hpw_size);
      break;
    case 49:  // accumulation tiles: (task, first row, first column)
      for (auto& t : P.acc_tiles) {
        v.push_back(t.x);
        v.push_back(t.y);
        v.push_back(t.z);
      }
      break;
    case 50:  // small matrix-product tiles: (task, first output)
      for (auto& t : P.mm_tiles) {
        v.push_back(t.x);
        v.push_back(t.y);
      }
      break;
    case 51:  // conversion tiles: (task, first element)
      for (auto& t : P.cvt_tiles) {
        v.push_back(t.x);
        v.push_back(t.y);
      }
      break;
    case 52:  // tensor-core hole-product groups: (A buf, A off, before, a, after, n, nchunks, image, members x 8)
      for (auto& g : P.hp_tc_groups) {
        v.push_back(g.A.buf);
        v.push_back(g.A.off);
        v.push_back(g.before);
        v.push_back(g.a);
        v.push_back(g.after);
        v.push_back(g.n);
        v.push_back(g.nchunks);
        v.push_back(g.img);
        for (int m = 0; m < qt::kHpTcMembers; ++m) v.push_back(m < g.n ? g.member[m] : -1);
      }
      break;
    case 53:  // tensor-core hole-product items: (group, range, first chunk, end chunk)
      for (auto& t : P.hp_tc_items) {
        v.push_back(t.x);
        v.push_back(t.y);
        v.push_back(t.z);
        v.push_back(t.w);
      }
      break;
    case 54:  // image pre-pass units: (group, chunk)
      for (auto& t : P.hp_tc_imgs) {
        v.push_back(t.x);
        v.push_back(t.y);
      }
      break;
    case 55:  // per stage: tensor-core hole-product items and image units (first, count, first, count)
      for (auto& st : P.stages) {
        v.push_back(st.hti0);
        v.push_back(st.nhti);
        v.push_back(st.htu0);
        v.push_back(st.nhtu);
      }
      break;
    case 56:  // B_OZ bytes
      v.push_back(P.oz_bytes);
      break;
    case 57:  // tensor-core accumulation items: (task, 128-row block, units before the item, 0)
      for (auto& t : P.acc_tc_items) {
        v.push_back(t.x);
        v.push_back(t.y);
        v.push_back(t.z);
        v.push_back(t.w);
      }
      break;
    case 58:  // image pre-pass units of the accumulations: (task, term)
      for (auto& t : P.acc_tc_imgs) {
        v.push_back(t.x);
        v.push_back(t.y);
      }
      break;
    case 59:  // per stage: accumulation items and image units (first, count, first, count, units)
      for (auto& st : P.stages) {
        v.push_back(st.ati0);
        v.push_back(st.nati);
        v.push_back(st.atu0);
        v.push_back(st.natu);
        v.push_back(st.atc_units);
      }
      break;
    case 60:  // accumulation tasks: byte offset of the term images in B_OZ (-1: classic)
      for (auto& t : P.acc) v.push_back(t.tc_img);
      break;
    default:
      break;
  }
}

// name of stage i of the plan (nullptr past the end)
const char* qtp_stage_name(void* h, int i) {
  const qt::Plan& P = static_cast<Handle*>(h)->plan;
  if (i < 0 || i >= (int)P.stages.size()) return nullptr;
  return P.stages[i].name;
}

static bool is_double_table(int what) { return (what >= 15 && what <= 17) || (what >= 30 && what <= 32); }

int64_t qtp_size(void* h, int what) {
  std::vector<int64_t> v;
  std::vector<double> dv;
  table(((Handle*)h)->plan, what, v, dv);
  return is_double_table(what) ? (int64_t)dv.size() : (int64_t)v.size();
}

void qtp_get(void* h, int what, void* out) {
  std::vector<int64_t> v;
  std::vector<double> dv;
  table(((Handle*)h)->plan, what, v, dv);
  if (is_double_table(what))
    std::memcpy(out, dv.data(), dv.size() * sizeof(double));
  else
    std::memcpy(out, v.data(), v.size() * sizeof(int64_t));
}

}  // extern "C"
