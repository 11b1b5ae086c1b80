// Host planner for one topology group.
//
// The reference evaluates, for every qMC sample, every topology and every initial
// sector, a recursive traversal of the configuration tree (src/topology_eval.jl:454-556):
// at an arc head it branches over the attachable interaction pairs, at an arc tail it
// continues only if operator_f has a block, and it multiplies operator x propagator
// blocks into a LazyMatrixProduct.  The shape of that tree does not depend on the sample
// times, so it is enumerated here once.  Two partial configurations whose futures are
// identical -- same position, initial sector, current sector, the same open arcs (tail
// position and pair type) and the same arcs still to come -- contribute with the same
// remaining factors; their partial products are summed and continued once.  The merged
// states form a DAG which is scheduled depth first into a linear program of small matrix
// instructions with an arena allocator.
//
// The hybridisation weight i*Delta_p(t_tail - t_head) of an arc is applied on its head
// edge (both times are known there) instead of at the tail, which lets states that differ
// only in the head positions of open arcs merge.  Results are sums of the same products in
// a different association, i.e. equal to the reference's up to rounding.
#include "qiw_plan.hpp"

#include <algorithm>
#include <cstring>
#include <map>
#include <set>
#include <functional>
#include <unordered_map>

#include "qiw.h"

namespace qiw {
namespace {

enum PosKind { PK_VAR = 0, PK_IDENT = 1, PK_OPER = 2 };

// Instruction flag bits set by the planner (bits 0-1 are set on upload from the coefficient):
// the product of a P multiply whose blocks have dimensions 1, 2 or 4 stays in registers for the
// out-edges emitted right after it.
constexpr uint8_t kFlagSrcReg = 4;    // OMUL / AXPY: the source is the register copy
constexpr uint8_t kFlagKeepReg = 8;   // PMUL: keep the product in registers
constexpr uint8_t kFlagNoStore = 16;  // PMUL: no instruction reads the product's arena copy
inline bool small_dim(int d) { return d == 1 || d == 2 || d == 4; }

struct Layout {
  int n = 0;
  std::vector<int> kind, op;     // per position
  std::vector<int> top_to_conf;  // topology vertex (0-based) -> position
  std::vector<int> zero_iv;      // interval pos -> pos+1 has zero length by construction
};

struct DNode {
  int pos, s0, s;
  int root_top = -1;             // >= 0: root of topology root_top (value parity * I or * O_B)
  int root_op = -1;
  double root_c = 1.0;
  int out_begin = 0, out_count = 0;  // out-edges: edges[out_begin .. out_begin + out_count)
  int n_in = 0;
  bool alive = false;
};

struct DEdge {
  int u, v, op, w;               // op: -1 identity; w: weight triple id or -1
};

// Most arcs a state can hold (open + future <= order), and the packing limit of a position,
// a sector or a pair index in one byte of an arc word.
constexpr int kMaxArcs = 16;

// A state: (s0, s, open arcs (tail, pair), future arcs (head, tail)).  Each arc is one word
// (first << 8 | second), so the ascending word order is the lexicographic order of the pairs.
struct State {
  int s0 = 0, s = 0;
  int n_open = 0, n_fut = 0;
  uint16_t open[kMaxArcs];
  uint16_t fut[kMaxArcs];

  static void insert(uint16_t *a, int *n, uint16_t v) {
    int i = *n;
    while (i > 0 && a[i - 1] > v) { a[i] = a[i - 1]; --i; }
    a[i] = v;
    ++*n;
  }
  static void erase(uint16_t *a, int *n, int k) {
    for (int i = k; i + 1 < *n; ++i) a[i] = a[i + 1];
    --*n;
  }
  bool operator==(const State &o) const {
    return s0 == o.s0 && s == o.s && n_open == o.n_open && n_fut == o.n_fut &&
           std::memcmp(open, o.open, n_open * sizeof(uint16_t)) == 0 &&
           std::memcmp(fut, o.fut, n_fut * sizeof(uint16_t)) == 0;
  }
};

struct StateHash {
  size_t operator()(const State &st) const {
    uint64_t h = 0x9e3779b97f4a7c15ull;
    auto mix = [&h](uint64_t v) {
      h ^= v + 0x9e3779b97f4a7c15ull + (h << 6) + (h >> 2);
      h *= 0xff51afd7ed558ccdull;
    };
    mix((uint64_t)(uint32_t)st.s0 << 32 | (uint32_t)st.s);
    mix((uint64_t)st.n_open << 8 | (uint64_t)st.n_fut);
    for (int i = 0; i < st.n_open; ++i) mix(st.open[i]);
    for (int i = 0; i < st.n_fut; ++i) mix((uint64_t)st.fut[i] << 16);
    return (size_t)(h ^ (h >> 33));
  }
};

struct Allocator {
  std::map<int64_t, int64_t> free_;  // offset -> size
  int64_t top = 0, peak = 0, live = 0;
  int64_t alloc(int64_t n) {
    for (auto it = free_.begin(); it != free_.end(); ++it) {
      if (it->second >= n) {
        int64_t off = it->first, sz = it->second;
        free_.erase(it);
        if (sz > n) free_[off + n] = sz - n;
        live += n;
        return off;
      }
    }
    int64_t off = top;
    top += n;
    peak = std::max(peak, top);
    live += n;
    return off;
  }
  void release(int64_t off, int64_t n) {
    live -= n;
    auto it = free_.emplace(off, n).first;
    auto nx = std::next(it);
    if (nx != free_.end() && it->first + it->second == nx->first) {
      it->second += nx->second;
      free_.erase(nx);
    }
    if (it != free_.begin()) {
      auto pv = std::prev(it);
      if (pv->first + pv->second == it->first) {
        pv->second += it->second;
        free_.erase(it);
        it = pv;
      }
    }
    if (it->first + it->second == top) {
      top = it->first;
      free_.erase(it);
    }
  }
};

struct Builder {
  const HostProblem &pb;
  const GroupSpec &g;
  const PlanOptions &opt;
  Layout L;
  // job ids in order of first use: (iv, s) -> Pm job, (head, tail, pair) -> W job (-1: none yet)
  std::vector<int> pm_slot, w_slot;
  std::vector<std::tuple<int, int, int>> w_list;
  std::vector<std::pair<int, int>> pm_list;
  std::string *err;

  Builder(const HostProblem &p, const GroupSpec &gs, const PlanOptions &o, std::string *e)
      : pb(p), g(gs), opt(o), err(e) {}

  int wid(int h, int t, int p) {
    const size_t k = ((size_t)h * L.n + t) * pb.n_pairs + p;
    if (w_slot.empty()) w_slot.assign((size_t)L.n * L.n * std::max(pb.n_pairs, 1), -1);
    if (w_slot[k] >= 0) return w_slot[k];
    const int id = (int)w_list.size();
    w_slot[k] = id;
    w_list.emplace_back(h, t, p);
    return id;
  }
  int pmid(int iv, int s) {
    const size_t k = (size_t)iv * pb.S + s;
    if (pm_slot.empty()) pm_slot.assign((size_t)L.n * pb.S, -1);
    if (pm_slot[k] >= 0) return pm_slot[k];
    const int id = (int)pm_list.size();
    pm_slot[k] = id;
    pm_list.emplace_back(iv, s);
    return id;
  }

  // Build the merged DAG for a set of roots (topology, s0).
  int build(const std::vector<std::pair<int, int>> &roots, std::vector<DNode> &nodes,
            std::vector<DEdge> &edges, std::vector<State> &states) {
    nodes.clear();
    edges.clear();
    states.clear();
    std::vector<std::unordered_map<State, int, StateHash>> maps(L.n);
    auto get = [&](int pos, const State &st) -> int {
      auto it = maps[pos].find(st);
      if (it != maps[pos].end()) return it->second;
      int id = (int)nodes.size();
      maps[pos].emplace(st, id);
      nodes.push_back(DNode{pos, st.s0, st.s});
      states.push_back(st);
      return id;
    };
    std::vector<int> layer;
    for (auto &r : roots) {
      int t = r.first, s0 = r.second;
      State st;
      st.s0 = s0;
      st.s = s0;
      for (auto &pr : g.tops[t]) {
        int x = pr.first, y = pr.second;
        if (x < 1 || y < 1 || x > 2 * g.order || y > 2 * g.order) {
          *err = "topology vertex out of range";
          return QIW_ERR_ARG;
        }
        int ph = L.top_to_conf[y - 1], ptl = L.top_to_conf[x - 1];
        if (!(ptl > ph)) {
          *err = "topology arc with tail not above head (pos_tail > pos_head violated)";
          return QIW_ERR_ARG;
        }
        State::insert(st.fut, &st.n_fut, (uint16_t)(ph << 8 | ptl));
      }
      int root_op = -1;
      if (L.kind[0] == PK_OPER) {
        root_op = L.op[0];
        int s1 = pb.target(root_op, s0);
        if (s1 < 0) continue;
        st.s = s1;
      }
      if (L.kind[0] == PK_VAR) {
        *err = "position 0 must hold a fixed node";
        return QIW_ERR_ARG;
      }
      int id = get(0, st);
      nodes[id].root_top = t;
      nodes[id].root_op = root_op;
      nodes[id].root_c = (double)g.parity[t];
      layer.push_back(id);
    }
    for (int pos = 1; pos < L.n; ++pos) {
      std::vector<int> next;
      for (int u : layer) {
        const State cur = states[u];
        nodes[u].out_begin = (int)edges.size();  // a state's out-edges are appended together
        auto add_edge = [&](const State &st, int op, int w) {
          int v = get(pos, st);
          edges.push_back(DEdge{u, v, op, w});
          nodes[u].out_count++;
          nodes[v].n_in++;
          if (nodes[v].n_in == 1) next.push_back(v);
        };
        if (L.kind[pos] == PK_IDENT) {
          add_edge(cur, -1, -1);
        } else if (L.kind[pos] == PK_OPER) {
          int t = pb.target(L.op[pos], cur.s);
          if (t >= 0) {
            State st = cur;
            st.s = t;
            add_edge(st, L.op[pos], -1);
          }
        } else {
          int fi = -1;
          for (int k = 0; k < cur.n_fut; ++k)
            if ((cur.fut[k] >> 8) == pos) fi = k;
          if (fi >= 0) {
            const int tail = cur.fut[fi] & 0xff;
            State base = cur;
            State::erase(base.fut, &base.n_fut, fi);
            for (int p = 0; p < pb.n_pairs; ++p) {
              int t = pb.target(pb.pair_op_i[p], cur.s);
              if (t < 0) continue;
              State st = base;
              st.s = t;
              State::insert(st.open, &st.n_open, (uint16_t)(tail << 8 | p));
              add_edge(st, pb.pair_op_i[p], wid(pos, tail, p));
            }
          } else {
            int oi = -1;
            for (int k = 0; k < cur.n_open; ++k)
              if ((cur.open[k] >> 8) == pos) oi = k;
            if (oi < 0) {
              *err = "configuration position is neither an arc head nor an arc tail";
              return QIW_ERR_ARG;
            }
            int p = cur.open[oi] & 0xff;
            int t = pb.target(pb.pair_op_f[p], cur.s);
            if (t >= 0) {
              State st = cur;
              st.s = t;
              State::erase(st.open, &st.n_open, oi);
              add_edge(st, pb.pair_op_f[p], -1);
            }
          }
        }
      }
      layer.swap(next);
    }
    // Leaves: s == s0 required (the reference asserts, src/topology_eval.jl:462-464).
    for (int u : layer) {
      if (nodes[u].s != nodes[u].s0) {
        *err = "A block off-diagonal contribution to a pseudo-particle propagator detected, "
               "try passing more 'symmetry_breakers' when constructing the local exact "
               "diagonalization object";
        return QIW_ERR_OFFDIAG;
      }
      nodes[u].alive = true;
    }
    // Backward liveness.
    for (int i = (int)nodes.size() - 1; i >= 0; --i) {
      if (nodes[i].alive) continue;
      for (int e = nodes[i].out_begin; e < nodes[i].out_begin + nodes[i].out_count; ++e)
        if (nodes[edges[e].v].alive) { nodes[i].alive = true; break; }
    }
    return 0;
  }

  double op_scalar(int op, int s, bool *ok) {
    int t = pb.target(op, s);
    *ok = false;
    if (t < 0 || pb.dims[t] != 1 || pb.dims[s] != 1) return 0.0;
    cd v = pb.op_vals[pb.op_valoff[(size_t)op * pb.S + s]];
    if (v.imag() != 0.0) return 0.0;
    *ok = true;
    return v.real();
  }

  bool diagP_group() const { return g.kind == QIW_GROUP_BARE; }

  // Schedule one batch into instructions; dynamic offsets relative to dyn_base.
  int schedule(std::vector<DNode> &nodes, std::vector<DEdge> &edges, std::vector<Instr> &ins,
               int64_t *peak, double *flops, const std::vector<int> &res_off) {
    Allocator al;
    int N = (int)nodes.size();
    std::vector<int64_t> slot(N, -1);
    std::vector<int> pending(N, 0);
    std::vector<int> n_out_alive(N, 0);
    for (auto &e : edges)
      if (nodes[e.u].alive && nodes[e.v].alive) { pending[e.v]++; n_out_alive[e.u]++; }
    auto dsz = [&](int u) { return (int64_t)pb.dims[nodes[u].s] * pb.dims[nodes[u].s0]; };
    std::vector<int> stack;
    for (int i = N - 1; i >= 0; --i)
      if (nodes[i].alive && nodes[i].pos == 0) stack.push_back(i);
    const int last = L.n - 1;
    bool all_scalar = opt.fuse_scalar;
    for (int t = 0; t < pb.S; ++t) all_scalar = all_scalar && pb.dims[t] == 1;
    double fl = 0.0;
    auto mk = [](uint8_t op) { Instr I; std::memset(&I, 0, sizeof(I)); I.op = op; I.w = -1; I.c = 1.0; return I; };
    std::vector<int> ready;
    while (!stack.empty()) {
      int u = stack.back();
      stack.pop_back();
      DNode &nu = nodes[u];
      int d = pb.dims[nu.s], d0 = pb.dims[nu.s0];
      if (nu.pos == last) {
        Instr I = mk(OP_LEAF);
        I.rows = (uint8_t)d;
        I.cols = (uint8_t)d0;
        I.src = (int32_t)slot[u];
        I.a = res_off[nu.s0];
        ins.push_back(I);
        fl += (double)d * d0;
        al.release(slot[u], dsz(u));
        continue;
      }
      // tmp = Pm[pos][s] * V_u; a zero-length interval (two fixed nodes at the same time) is
      // the identity: no P block, tmp is V_u itself (or c * identity for an identity root)
      const bool zero_iv = !L.zero_iv.empty() && L.zero_iv[nu.pos];
      const bool ident_root = nu.root_top >= 0 && nu.root_op < 0;
      int pmj = zero_iv ? -1 : pmid(nu.pos, nu.s);
      // 1x1 problems: a P multiply whose one live out-edge is an AXPY (not the alias case, where
      // the product already is V_v) becomes one PMAXPY; the product is rounded as before.
      if (all_scalar && !zero_iv && !ident_root && n_out_alive[u] == 1) {
        int fe = -1;
        for (int e = nu.out_begin; e < nu.out_begin + nu.out_count; ++e)
          if (nodes[edges[e].v].alive) { fe = e; break; }
        const DEdge &E = edges[fe];
        const int v = E.v;
        const bool alias = E.op < 0 && E.w < 0 && pending[v] == 1 && slot[v] < 0;
        bool ok = E.op < 0;
        double sc = 1.0;
        if (!ok && opt.fold_scalar_ops) sc = op_scalar(E.op, nu.s, &ok);
        if (!alias && ok) {
          int64_t src = slot[u];
          if (nu.root_top >= 0) {  // operator root: materialise parity * O_B
            src = al.alloc(1);
            Instr I = mk(OP_LOADC);
            I.rows = 1;
            I.cols = 1;
            I.dst = (int32_t)src;
            I.a = (int32_t)pb.op_valoff[(size_t)nu.root_op * pb.S + nu.s0];
            I.c = nu.root_c;
            ins.push_back(I);
          }
          al.release(src, 1);
          const bool acc = slot[v] >= 0;
          if (!acc) slot[v] = al.alloc(1);
          Instr I = mk(OP_PMAXPY);
          I.rows = 1;
          I.inner = 1;
          I.cols = 1;
          I.acc = acc;
          I.dst = (int32_t)slot[v];
          I.src = (int32_t)src;
          I.a = pmj;
          I.w = E.w;
          I.c = (E.op < 0) ? 1.0 : sc;
          ins.push_back(I);
          fl += (diagP_group() ? 1.0 : 2.0) + ((E.w >= 0 || I.c != 1.0 ? 1 : 0) + (acc ? 1 : 0));
          if (--pending[v] == 0) stack.push_back(v);
          continue;
        }
      }
      int64_t tmp = (zero_iv && !ident_root) ? -1 : al.alloc((int64_t)d * d0);
      bool diagP = (g.kind == QIW_GROUP_BARE);
      int64_t pmul_at = -1;   // index of this node's P multiply when its product may stay in registers
      if (ident_root && zero_iv) {
        Instr I = mk(OP_LOADI);
        I.rows = (uint8_t)d;
        I.cols = (uint8_t)d;
        I.dst = (int32_t)tmp;
        I.c = nu.root_c;
        ins.push_back(I);
      } else if (ident_root) {
        Instr I = mk(OP_LOADP);
        I.rows = (uint8_t)d;
        I.cols = (uint8_t)d;
        I.inner = diagP ? 1 : 0;
        I.dst = (int32_t)tmp;
        I.a = pmj;  // resolved to an arena offset later
        I.c = nu.root_c;
        ins.push_back(I);
        fl += (double)d * d;
      } else {
        int64_t src = slot[u];
        if (nu.root_top >= 0) {  // operator root: materialise parity * O_B block
          src = al.alloc((int64_t)d * d0);
          Instr I = mk(OP_LOADC);
          I.rows = (uint8_t)d;
          I.cols = (uint8_t)d0;
          I.dst = (int32_t)src;
          I.a = (int32_t)pb.op_valoff[(size_t)nu.root_op * pb.S + nu.s0];
          I.c = nu.root_c;
          ins.push_back(I);
        }
        if (zero_iv) {
          tmp = src;
        } else {
          Instr I = mk(diagP ? OP_PMULD : OP_PMUL);
          I.rows = (uint8_t)d;
          I.inner = (uint8_t)d;
          I.cols = (uint8_t)d0;
          I.dst = (int32_t)tmp;
          I.src = (int32_t)src;
          I.a = pmj;
          ins.push_back(I);
          fl += diagP ? (double)d * d0 : 2.0 * d * d * d0;
          al.release(src, (int64_t)d * d0);
          if (!diagP && !all_scalar && small_dim(d) && small_dim(d0)) pmul_at = (int64_t)ins.size() - 1;
        }
      }
      bool tmp_taken = false, tmp_read = false;   // the arena copy of tmp is needed / read
      ready.clear();
      for (int e = nu.out_begin; e < nu.out_begin + nu.out_count; ++e) {
        const DEdge &E = edges[e];
        if (!nodes[E.v].alive) continue;
        int v = E.v;
        int dv = pb.dims[nodes[v].s];
        if (E.op < 0 && E.w < 0 && n_out_alive[u] == 1 && pending[v] == 1 && slot[v] < 0) {
          slot[v] = tmp;  // alias: V_v is tmp itself
          tmp_taken = true;
          tmp_read = true;
        } else {
          bool acc = slot[v] >= 0;
          if (!acc) slot[v] = al.alloc(dsz(v));
          bool ok = false;
          double sc = 1.0;
          if (E.op >= 0 && opt.fold_scalar_ops) sc = op_scalar(E.op, nu.s, &ok);
          if (E.op < 0 || ok) {
            Instr I = mk(OP_AXPY);
            I.rows = (uint8_t)dv;
            I.cols = (uint8_t)d0;
            I.acc = acc;
            I.dst = (int32_t)slot[v];
            I.src = (int32_t)tmp;
            I.w = E.w;
            I.c = (E.op < 0) ? 1.0 : sc;
            if (pmul_at >= 0 && small_dim(dv)) I.flags |= kFlagSrcReg;
            else tmp_read = true;
            ins.push_back(I);
            fl += (double)dv * d0 * ((E.w >= 0 || I.c != 1.0 ? 1 : 0) + (acc ? 1 : 0));
          } else {
            Instr I = mk(OP_OMUL);
            I.rows = (uint8_t)dv;
            I.inner = (uint8_t)d;
            I.cols = (uint8_t)d0;
            I.acc = acc;
            I.dst = (int32_t)slot[v];
            I.src = (int32_t)tmp;
            I.a = (int32_t)pb.op_valoff[(size_t)E.op * pb.S + nu.s];
            I.w = E.w;
            if (pmul_at >= 0 && small_dim(dv)) I.flags |= kFlagSrcReg;
            else tmp_read = true;
            ins.push_back(I);
            fl += 2.0 * dv * d * d0 + (E.w >= 0 ? (double)dv * d0 : 0.0);
          }
        }
        if (--pending[v] == 0) ready.push_back(v);
      }
      if (pmul_at >= 0) {   // the out-edges above read the product from registers
        ins[pmul_at].flags |= kFlagKeepReg;
        if (!tmp_read) ins[pmul_at].flags |= kFlagNoStore;
      }
      if (!tmp_taken) al.release(tmp, (int64_t)d * d0);
      for (auto it = ready.rbegin(); it != ready.rend(); ++it) stack.push_back(*it);
    }
    *peak = al.peak;
    *flops += fl;
    return 0;
  }



  // Number of configurations and flops of the reference's per-topology tree traversal
  // with LazyMatrixProduct caching (complex arithmetic): a pushed factor is multiplied
  // once if some leaf lies below it; each leaf adds weight * product into the result.
  void tree_count(double *flops, int64_t *leaves) {
    double fl = 0.0;
    int64_t nl = 0;
    const int n = L.n;
    // node matrices of all positions >= 1 (src/topology_eval.jl:376-388)
    for (int pos = 1; pos < n; ++pos) {
      std::vector<int> ops;
      if (L.kind[pos] == PK_VAR)
        for (int p = 0; p < pb.n_pairs; ++p) { ops.push_back(pb.pair_op_i[p]); ops.push_back(pb.pair_op_f[p]); }
      else ops.push_back(L.kind[pos] == PK_OPER ? L.op[pos] : pb.identity_op);
      for (int op : ops)
        for (int s = 0; s < pb.S; ++s) {
          int t = pb.target(op, s);
          if (t >= 0) fl += 8.0 * pb.dims[t] * pb.dims[s] * pb.dims[s];
        }
    }
    for (size_t t = 0; t < g.tops.size(); ++t) {
      std::vector<int> head_tail(n, -1), is_tail(n, 0), arc_of(n, -1);
      for (size_t a = 0; a < g.tops[t].size(); ++a) {
        int ph = L.top_to_conf[g.tops[t][a].second - 1], pt = L.top_to_conf[g.tops[t][a].first - 1];
        head_tail[ph] = pt;
        is_tail[pt] = 1;
        arc_of[ph] = arc_of[pt] = (int)a;
      }
      std::vector<int> sel(g.tops[t].size(), -1);
      for (int s0 = 0; s0 < pb.S; ++s0) {
        // returns number of leaves below; adds flops of factors with leaves below
        std::function<int64_t(int, int, int)> rec = [&](int pos, int s, int depth) -> int64_t {
          if (pos >= n) {
            if (s == s0) { fl += 8.0 * pb.dims[s0] * pb.dims[s0]; return 1; }
            return 0;
          }
          auto push = [&](int sn, int inner) -> double {
            return depth == 0 ? 0.0 : 8.0 * pb.dims[sn] * inner * pb.dims[s0];
          };
          int64_t total = 0;
          if (L.kind[pos] == PK_IDENT) {
            if (pos == 0) return rec(pos + 1, s, depth);
            int64_t c = rec(pos + 1, s, depth + 1);
            if (c) fl += push(s, pb.dims[s]);
            return c;
          }
          if (L.kind[pos] == PK_OPER) {
            int sn = pb.target(L.op[pos], s);
            if (sn < 0) return 0;
            int64_t c = rec(pos + 1, sn, depth + 1);
            if (c) fl += push(sn, pb.dims[s]);
            return c;
          }
          if (head_tail[pos] >= 0) {
            for (int p = 0; p < pb.n_pairs; ++p) {
              int sn = pb.target(pb.pair_op_i[p], s);
              if (sn < 0) continue;
              sel[arc_of[pos]] = p;
              int64_t c = rec(pos + 1, sn, depth + 1);
              if (c) fl += push(sn, pb.dims[s]);
              total += c;
            }
            return total;
          }
          int p = sel[arc_of[pos]];
          int sn = pb.target(pb.pair_op_f[p], s);
          if (sn < 0) return 0;
          int64_t c = rec(pos + 1, sn, depth + 1);
          if (c) fl += push(sn, pb.dims[s]) + 6.0;
          return c;
        };
        nl += rec(0, s0, 0);
      }
    }
    *flops = fl;
    *leaves = nl;
  }

  int setup_layout(Plan *out) {
    const int k = g.order;
    int n, d_before = 0, d_after = 0;
    if (g.kind == QIW_GROUP_BARE) {
      n = 2 * k + 2;
    } else if (g.kind == QIW_GROUP_BOLD || g.kind == QIW_GROUP_CORRELATOR) {
      n = 2 * k + 3;
      if (k > 0) {
        d_after = g.n_pts_after;
        d_before = 2 * k - g.n_pts_after;
        if (d_after < 1 || d_before < 0) {
          *err = "n_pts_after must lie in 1:2*order";
          return QIW_ERR_ARG;
        }
      }
    } else if (g.kind == QIW_GROUP_SIGMA) {
      // PairNode(t_i) ... PairNode(t_f) (src/inchworm.jl:560-566), framed by identities at the
      // same times: the two end intervals have zero length and are skipped by the scheduler
      if (k < 1) {
        *err = "self-energy groups start at order 1";
        return QIW_ERR_ARG;
      }
      n = 2 * k + 2;
    } else {
      *err = "unknown group kind";
      return QIW_ERR_ARG;
    }
    if (n > kMaxNodes || 2 * k > kMaxDim) {
      *err = "expansion order too large for this build";
      return QIW_ERR_UNSUPPORTED;
    }
    L.n = n;
    L.kind.assign(n, PK_VAR);
    L.op.assign(n, -1);
    out->n_fixed = 0;
    auto fix = [&](int pos, int kind, int op, int tsel) {
      L.kind[pos] = kind;
      L.op[pos] = op;
      out->fixed_pos[out->n_fixed] = pos;
      out->fixed_time[out->n_fixed] = tsel;
      out->n_fixed++;
    };
    std::vector<int> time_fixed(n, 0);
    L.zero_iv.assign(n, 0);
    if (g.kind == QIW_GROUP_BARE) {
      fix(0, PK_IDENT, -1, T_I);
      fix(n - 1, PK_IDENT, -1, T_F);
    } else if (g.kind == QIW_GROUP_SIGMA) {
      fix(0, PK_IDENT, -1, T_I);
      fix(n - 1, PK_IDENT, -1, T_F);
      // pair vertices with fixed times: they stay pair positions of the topology
      out->fixed_pos[out->n_fixed] = 1;
      out->fixed_time[out->n_fixed++] = T_I;
      out->fixed_pos[out->n_fixed] = n - 2;
      out->fixed_time[out->n_fixed++] = T_F;
      time_fixed[1] = time_fixed[n - 2] = 1;
      L.zero_iv[0] = L.zero_iv[n - 2] = 1;
    } else if (g.kind == QIW_GROUP_BOLD) {
      fix(0, PK_IDENT, -1, T_I);
      fix(d_before + 1, PK_IDENT, -1, T_W);
      fix(n - 1, PK_IDENT, -1, T_F);
    } else {
      if (g.corr_A < 0 || g.corr_B < 0 || g.corr_A >= pb.n_ops || g.corr_B >= pb.n_ops) {
        *err = "correlator operator index out of range";
        return QIW_ERR_ARG;
      }
      fix(0, PK_OPER, g.corr_B, T_I);
      fix(d_before + 1, PK_OPER, g.corr_A, T_W);
      fix(n - 1, PK_IDENT, -1, T_F);
    }
    // src/topology_eval.jl:269-275: both maps run over positions in reverse order.
    L.top_to_conf.clear();
    out->var_pos.clear();
    for (int pos = n - 1; pos >= 0; --pos)
      if (L.kind[pos] == PK_VAR) {
        L.top_to_conf.push_back(pos);
        if (!time_fixed[pos]) out->var_pos.push_back(pos);
      }
    out->kind = g.kind;
    out->order = k;
    out->n_nodes = n;
    out->D = (int)out->var_pos.size();
    out->d_before = d_before;
    out->d_after = d_after;
    out->use_bold = g.kind != QIW_GROUP_BARE;
    return 0;
  }
};

void append_bytes(std::string *k, const void *p, size_t n) { k->append(reinterpret_cast<const char *>(p), n); }

template <typename T>
void append_vec(std::string *k, const std::vector<T> &v) {
  const uint64_t n = v.size();
  append_bytes(k, &n, sizeof(n));
  if (n) append_bytes(k, v.data(), n * sizeof(T));
}

}  // namespace

std::string plan_key(const HostProblem &hp, const GroupSpec &gs) {
  std::string k;
  append_bytes(&k, &hp.S, sizeof(hp.S));
  append_vec(&k, hp.dims);
  append_bytes(&k, &hp.n_ops, sizeof(hp.n_ops));
  append_vec(&k, hp.op_target);
  append_vec(&k, hp.op_valoff);
  append_vec(&k, hp.op_vals);
  append_bytes(&k, &hp.identity_op, sizeof(hp.identity_op));
  append_bytes(&k, &hp.n_pairs, sizeof(hp.n_pairs));
  append_vec(&k, hp.pair_op_i);
  append_vec(&k, hp.pair_op_f);
  const int g[5] = {gs.kind, gs.order, gs.n_pts_after, gs.corr_A, gs.corr_B};
  append_bytes(&k, g, sizeof(g));
  for (const auto &t : gs.tops) append_vec(&k, t);
  append_vec(&k, gs.parity);
  return k;
}

int plan_group(const HostProblem &pb, const GroupSpec &g, const PlanOptions &opt, Plan *out,
               std::string *err) {
  *out = Plan();
  if ((int)g.tops.size() != (int)g.parity.size()) {
    *err = "topology / parity count mismatch";
    return QIW_ERR_ARG;
  }
  for (auto &t : g.tops)
    if ((int)t.size() != g.order) {
      *err = "topology order mismatch";
      return QIW_ERR_ARG;
    }
  for (int s = 0; s < pb.S; ++s)
    if (pb.dims[s] > 255) {
      *err = "sector dimension above 255";
      return QIW_ERR_UNSUPPORTED;
    }
  Builder B(pb, g, opt, err);
  int rc = B.setup_layout(out);
  if (rc) return rc;
  if (g.order > kMaxArcs || B.L.n > 256 || pb.n_pairs > 256) {
    *err = "group beyond the planner's packing limits (order <= 16, <= 256 positions and pairs)";
    return QIW_ERR_UNSUPPORTED;
  }
  std::vector<int> res_off(pb.S);
  int ro = 0;
  for (int s = 0; s < pb.S; ++s) { res_off[s] = ro; ro += pb.dims[s] * pb.dims[s]; }
  out->res_size = ro;

  // Upper bound of the fixed (Pm + W) part of the arena, for the batch budget.
  int64_t sumd2 = 0;
  for (int s = 0; s < pb.S; ++s) sumd2 += (int64_t)pb.dims[s] * pb.dims[s];
  std::set<std::pair<int, int>> arcs;  // distinct (head, tail) positions over all topologies
  for (auto &t : g.tops)
    for (auto &pr : t) {
      int x = pr.first, y = pr.second;
      if (x >= 1 && y >= 1 && x <= 2 * g.order && y <= 2 * g.order)
        arcs.emplace(B.L.top_to_conf[y - 1], B.L.top_to_conf[x - 1]);
    }
  int64_t fixed_bound = (int64_t)(out->n_nodes - 1) * sumd2 + (int64_t)arcs.size() * pb.n_pairs;
  int64_t dyn_budget = std::max<int64_t>(opt.arena_budget - fixed_bound, 64);

  // One root list per initial sector: different s0 never merge, so each s0 is an
  // independent batch (a separately schedulable unit of work) at no extra cost.
  std::vector<std::vector<std::pair<int, int>>> s0_roots(pb.S);
  for (int t = 0; t < (int)g.tops.size(); ++t)
    for (int s0 = 0; s0 < pb.S; ++s0) s0_roots[s0].emplace_back(t, s0);

  std::vector<Instr> ins;
  int64_t dyn_peak = 0;
  double flops = 0.0;
  int64_t dag_nodes = 0;
  int n_batches = 0;
  std::vector<DNode> nodes;
  std::vector<DEdge> edges;
  std::vector<State> states;
  // Recursive batch planner: merge as much as the working-set budget allows.
  std::function<int(const std::vector<std::pair<int, int>> &)> plan_roots =
      [&](const std::vector<std::pair<int, int>> &roots) -> int {
    if (roots.empty()) return 0;
    int r = B.build(roots, nodes, edges, states);
    if (r) return r;
    std::vector<Instr> bi;
    int64_t peak = 0;
    double fl = 0.0;
    r = B.schedule(nodes, edges, bi, &peak, &fl, res_off);
    if (r) return r;
    const bool too_long = (opt.max_batch_flops > 0.0 && fl > opt.max_batch_flops) ||   // one thread's serial work
                          (opt.max_batch_instrs > 0 && (int64_t)bi.size() > opt.max_batch_instrs);
    if ((peak > dyn_budget || too_long) && roots.size() > 1) {
      // split: by initial sector first, then by topology halves
      std::vector<std::pair<int, int>> a, b;
      int s_first = roots.front().second;
      bool one_s0 = std::all_of(roots.begin(), roots.end(), [&](auto &x) { return x.second == s_first; });
      if (!one_s0) {
        std::vector<int> s0s;
        for (auto &x : roots) s0s.push_back(x.second);
        std::sort(s0s.begin(), s0s.end());
        s0s.erase(std::unique(s0s.begin(), s0s.end()), s0s.end());
        std::vector<int> lo(s0s.begin(), s0s.begin() + s0s.size() / 2);
        for (auto &x : roots) (std::binary_search(lo.begin(), lo.end(), x.second) ? a : b).push_back(x);
      } else {
        a.assign(roots.begin(), roots.begin() + roots.size() / 2);
        b.assign(roots.begin() + roots.size() / 2, roots.end());
      }
      r = plan_roots(a);
      if (r) return r;
      return plan_roots(b);
    }
    if (peak > dyn_budget) {
      *err = "a single (topology, sector) configuration tree exceeds the per-sample working-set budget";
      return QIW_ERR_MEMORY;
    }
    for (auto &nd : nodes) dag_nodes += nd.alive ? 1 : 0;
    if (bi.empty()) return 0;
    out->batch_begin.push_back((int32_t)ins.size());
    out->batch_flops.push_back(fl);
    ins.insert(ins.end(), bi.begin(), bi.end());
    dyn_peak = std::max(dyn_peak, peak);
    flops += fl;
    n_batches++;
    return 0;
  };
  for (int s0 = 0; s0 < pb.S; ++s0) {
    rc = plan_roots(s0_roots[s0]);
    if (rc) return rc;
  }
  out->batch_begin.push_back((int32_t)ins.size());

  // Resolve arena offsets: [Pm jobs][W jobs][dynamic].
  int64_t off = 0;
  std::vector<int32_t> pm_off(B.pm_list.size());
  for (size_t j = 0; j < B.pm_list.size(); ++j) {
    int s = B.pm_list[j].second;
    pm_off[j] = (int32_t)off;
    out->pm.push_back(PmJob{(int16_t)B.pm_list[j].first, (int16_t)s, (int32_t)off});
    off += (g.kind == QIW_GROUP_BARE) ? pb.dims[s] : (int64_t)pb.dims[s] * pb.dims[s];
    flops += (g.kind == QIW_GROUP_BARE) ? pb.dims[s] : 3.0 * pb.dims[s] * pb.dims[s];
  }
  std::vector<int32_t> w_off(B.w_list.size());
  for (size_t j = 0; j < B.w_list.size(); ++j) {
    w_off[j] = (int32_t)off;
    out->wj.push_back(WJob{(int16_t)std::get<0>(B.w_list[j]), (int16_t)std::get<1>(B.w_list[j]),
                           (int16_t)std::get<2>(B.w_list[j]), 0, (int32_t)off});
    off += 1;
    flops += 3.0;
  }
  int64_t dyn_base = off;
  for (auto &I : ins) {
    switch (I.op) {
      case OP_LOADP: I.a = pm_off[I.a]; I.dst += (int32_t)dyn_base; break;
      case OP_PMUL:
      case OP_PMULD:
      case OP_PMAXPY: I.a = pm_off[I.a]; I.dst += (int32_t)dyn_base; I.src += (int32_t)dyn_base; break;
      case OP_LOADC:
      case OP_LOADI: I.dst += (int32_t)dyn_base; break;
      case OP_OMUL:
      case OP_AXPY: I.dst += (int32_t)dyn_base; I.src += (int32_t)dyn_base; break;
      case OP_LEAF: I.src += (int32_t)dyn_base; break;
      default: break;
    }
    if (I.w >= 0) I.w = w_off[I.w];
  }
  out->ins = std::move(ins);
  out->arena = dyn_base + dyn_peak;
  out->dag_nodes = dag_nodes;
  out->flops = flops;
  out->n_batches = n_batches;
  B.tree_count(&out->tree_flops, &out->tree_leaves);
  return 0;
}

}  // namespace qiw

namespace qiw {

int host_problem_from_desc(const void *pdv, HostProblem *hpo, std::string *err) {
  const qiw_problem_desc *d = static_cast<const qiw_problem_desc *>(pdv);
  HostProblem &hp = *hpo;
  hp = HostProblem();
  if (d->n_sectors <= 0 || !d->sector_dims || d->n_ops <= 0 || !d->op_n_blocks || !d->op_blocks ||
      !d->op_value_offset || !d->op_values || d->n_pairs < 0 || (d->n_pairs > 0 && !d->pair_ops)) {
    *err = "missing or invalid problem field";
    return QIW_ERR_ARG;
  }
  hp.S = d->n_sectors;
  hp.dims.assign(d->sector_dims, d->sector_dims + hp.S);
  for (int s = 0; s < hp.S; ++s)
    if (hp.dims[s] <= 0 || hp.dims[s] > 255) {
      *err = "sector dimension out of range";
      return QIW_ERR_ARG;
    }
  hp.n_ops = d->n_ops;
  hp.op_target.assign((size_t)hp.n_ops * hp.S, -1);
  hp.op_valoff.assign((size_t)hp.n_ops * hp.S, -1);
  int64_t k = 0, max_val = 0;
  for (int o = 0; o < hp.n_ops; ++o) {
    if (d->op_n_blocks[o] < 0) {
      *err = "negative block count";
      return QIW_ERR_ARG;
    }
    for (int b = 0; b < d->op_n_blocks[o]; ++b, ++k) {
      int si = d->op_blocks[2 * k], sf = d->op_blocks[2 * k + 1];
      int64_t off = d->op_value_offset[k];
      if (si < 0 || si >= hp.S || sf < 0 || sf >= hp.S || off < 0) {
        *err = "operator block index out of range";
        return QIW_ERR_ARG;
      }
      if (hp.op_target[(size_t)o * hp.S + si] >= 0) {
        *err = "operator is not a SectorBlockMatrix (two blocks in one column)";
        return QIW_ERR_ARG;
      }
      hp.op_target[(size_t)o * hp.S + si] = sf;
      hp.op_valoff[(size_t)o * hp.S + si] = off;
      max_val = std::max<int64_t>(max_val, off + (int64_t)hp.dims[si] * hp.dims[sf]);
    }
  }
  hp.op_vals.resize(max_val);
  for (int64_t i = 0; i < max_val; ++i) hp.op_vals[i] = cd(d->op_values[2 * i], d->op_values[2 * i + 1]);
  if (d->identity_op < 0 || d->identity_op >= hp.n_ops) {
    *err = "identity_op out of range";
    return QIW_ERR_ARG;
  }
  hp.identity_op = d->identity_op;
  hp.n_pairs = d->n_pairs;
  hp.pair_op_i.resize(hp.n_pairs);
  hp.pair_op_f.resize(hp.n_pairs);
  for (int p = 0; p < hp.n_pairs; ++p) {
    int oi = d->pair_ops[2 * p], of = d->pair_ops[2 * p + 1];
    if (oi < 0 || oi >= hp.n_ops || of < 0 || of >= hp.n_ops) {
      *err = "pair operator out of range";
      return QIW_ERR_ARG;
    }
    hp.pair_op_i[p] = oi;
    hp.pair_op_f[p] = of;
  }
  return 0;
}

int group_spec_from_desc(const void *gdv, GroupSpec *gs, std::string *err) {
  const qiw_group_desc *d = static_cast<const qiw_group_desc *>(gdv);
  if (d->order < 0 || d->n_topologies < 0 || (d->order > 0 && d->n_topologies > 0 && !d->top_pairs) ||
      (d->n_topologies > 0 && !d->top_parity)) {
    *err = "invalid group descriptor";
    return QIW_ERR_ARG;
  }
  *gs = GroupSpec();
  gs->kind = d->kind;
  gs->order = d->order;
  gs->n_pts_after = d->n_pts_after;
  gs->corr_A = d->corr_A_op;
  gs->corr_B = d->corr_B_op;
  gs->tops.resize(d->n_topologies);
  gs->parity.resize(d->n_topologies);
  for (int t = 0; t < d->n_topologies; ++t) {
    for (int a = 0; a < d->order; ++a)
      gs->tops[t].emplace_back(d->top_pairs[(size_t)(t * d->order + a) * 2],
                               d->top_pairs[(size_t)(t * d->order + a) * 2 + 1]);
    gs->parity[t] = d->top_parity[t];
  }
  return 0;
}

}  // namespace qiw
