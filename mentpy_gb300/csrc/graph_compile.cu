// Native plan compiler: open graph + measurements -> window-plan tables.
//
// Restates, on integer node indices, what MBQCircuit and the simulators'
// constructors compute on networkx graphs:
//   * the causal flow layers, the layer-by-layer search of Mhalla and Perdrix
//     in the form of mentpy/mbqc/flow.py:115-188 (find_cflow);
//   * the measurement order, MBQCircuit.calculate_order
//     (mentpy/mbqc/mbqcircuit.py:390-422);
//   * the window schedule, the in-place bit assignment and the per-step
//     tables, the window bookkeeping of NumpySimulatorSV/NumpySimulatorDM
//     (np_simulator_sv.py:61-128,207-223,278-297; np_simulator_dm.py:47-115,
//     267-283), in the in-place form the kernels run (the qubit entering at
//     step k takes bit k mod w).
//
// find_cflow walks its frontier in Python set order, and two frontier nodes
// that compete for one candidate make the result depend on that order.  This
// compiler detects every such layer (a candidate shared by two frontier
// nodes) and then returns MBQC_E_UNSUPPORTED, so that the caller uses the
// Python compiler, which iterates real Python sets.  Without a shared
// candidate the layers do not depend on the iteration order.
#include <cstdint>
#include <cstring>
#include <string>
#include <unordered_map>
#include <vector>

#include "dispatch.h"

namespace mbqc {

namespace {

constexpr uint32_t kDeadBit = 0x80000000u;

struct Graph {
  int n = 0;
  std::vector<std::vector<int>> adj;  // neighbour indices
};

// Causal-flow layers (flow.py:115-188).  Returns 1 when a flow exists, 0 when
// not, -1 when the search met a candidate shared by two frontier nodes.
int flow_layers(const Graph &g, const std::vector<int> &inputs, const std::vector<int> &outputs,
                std::vector<int> &layer) {
  const int n = g.n;
  layer.assign(n, 0);
  std::vector<int> past(n, 0);
  std::vector<char> is_out(n, 0), is_in(n, 0), orig_out(n, 0);
  for (int v : outputs) is_out[v] = orig_out[v] = 1;
  for (int v : inputs) is_in[v] = 1;
  int n_succ = 0;

  std::vector<int> frontier;
  std::vector<char> in_front(n, 0);
  for (int v : outputs) {
    if (is_in[v]) continue;
    int c = 0;
    for (int u : g.adj[v])
      if (!orig_out[u]) ++c;
    past[v] = c;
    if (c == 1 && !in_front[v]) {
      in_front[v] = 1;
      frontier.push_back(v);
    }
  }

  std::vector<int> claim(n, -1);  // frontier node that has u as a candidate, this layer
  std::vector<char> in_next(n, 0);
  for (int k = 1;; ++k) {
    // shared-candidate check: every non-output neighbour of a frontier node
    // with a non-empty candidate set must belong to one frontier node only
    for (int v : frontier)
      for (int u : g.adj[v])
        if (!is_out[u]) {
          if (claim[u] != -1 && claim[u] != v) return -1;
          claim[u] = v;
        }
    std::vector<int> next;
    for (int v : frontier) {
      int cand = -1, nc = 0;
      for (int u : g.adj[v])
        if (!is_out[u]) {
          cand = u;
          ++nc;
        }
      if (nc != 1) continue;
      const int u = cand;
      layer[u] = k;
      ++n_succ;
      is_out[u] = 1;
      if (!is_in[u]) {
        int c = 0;
        for (int x : g.adj[u])
          if (!is_out[x]) ++c;
        past[u] = c;
        if (c == 1 && !in_next[u]) {
          in_next[u] = 1;
          next.push_back(u);
        }
      }
      for (int w : g.adj[u])
        if (past[w] > 0) {
          --past[w];
          if (past[w] == 1 && !in_next[w]) {
            in_next[w] = 1;
            next.push_back(w);
          }
        }
    }
    for (int v : frontier)
      for (int u : g.adj[v]) claim[u] = -1;
    for (int v : next) in_next[v] = 0;
    for (int v : frontier) in_front[v] = 0;
    if (next.empty()) break;
    frontier.swap(next);
  }
  return n_succ == n - (int)outputs.size() ? 1 : 0;
}

}  // namespace

}  // namespace mbqc

using namespace mbqc;

extern "C" {

int mbqc_compile_graph(const mbqc_graph_desc *d, mbqc_plan_tables *t) {
  if (!d || !t) return fail(MBQC_E_INVALID, "compile_graph: null argument");
  const int n = d->n_nodes;
  if (n <= 0 || !d->nodes) return fail(MBQC_E_INVALID, "compile_graph: no nodes");
  if (d->kind != 0 && d->kind != 1) return fail(MBQC_E_INVALID, "compile_graph: kind must be 0 (sv) or 1 (dm)");
  if (d->n_edges < 0 || (d->n_edges > 0 && !d->edges)) return fail(MBQC_E_INVALID, "compile_graph: edges");
  if (!d->plane || !d->trainable || !d->angle) return fail(MBQC_E_INVALID, "compile_graph: node arrays");
  if (d->n_inputs < 0 || d->n_outputs < 0 || (d->n_inputs && !d->inputs) ||
      (d->n_outputs && !d->outputs))
    return fail(MBQC_E_INVALID, "compile_graph: inputs/outputs");

  // labels -> graph-order indices: a direct table for small non-negative
  // labels (the usual 0..n-1), a hash map otherwise
  int32_t lo = d->nodes[0], hi = d->nodes[0];
  for (int i = 1; i < n; ++i) {
    lo = d->nodes[i] < lo ? d->nodes[i] : lo;
    hi = d->nodes[i] > hi ? d->nodes[i] : hi;
  }
  const bool direct = lo >= 0 && (int64_t)hi < 4 * (int64_t)n + 64;
  std::vector<int> table;
  std::unordered_map<int32_t, int> idx;
  if (direct) {
    table.assign((size_t)hi + 1, -1);
    for (int i = 0; i < n; ++i) {
      if (table[d->nodes[i]] != -1) return fail(MBQC_E_INVALID, "compile_graph: duplicate node");
      table[d->nodes[i]] = i;
    }
  } else {
    idx.reserve((size_t)n * 2);
    for (int i = 0; i < n; ++i)
      if (!idx.emplace(d->nodes[i], i).second) return fail(MBQC_E_INVALID, "compile_graph: duplicate node");
  }
  auto index_of = [&](int32_t lbl, int &out) {
    if (direct) {
      if (lbl < 0 || lbl > hi || table[lbl] < 0) return false;
      out = table[lbl];
      return true;
    }
    auto it = idx.find(lbl);
    if (it == idx.end()) return false;
    out = it->second;
    return true;
  };
  Graph g;
  g.n = n;
  g.adj.assign(n, {});
  for (int e = 0; e < d->n_edges; ++e) {
    int a, b;
    if (!index_of(d->edges[2 * e], a) || !index_of(d->edges[2 * e + 1], b))
      return fail(MBQC_E_INVALID, "compile_graph: edge %d names an unknown node", e);
    if (a == b) return fail(MBQC_E_UNSUPPORTED, "compile_graph: self loop");
    bool dup = false;
    for (int x : g.adj[a]) dup |= (x == b);
    if (dup) continue;  // a graph, not a multigraph
    g.adj[a].push_back(b);
    g.adj[b].push_back(a);
  }
  std::vector<int> inputs(d->n_inputs), outputs(d->n_outputs);
  std::vector<char> is_output(n, 0);
  for (int i = 0; i < d->n_inputs; ++i)
    if (!index_of(d->inputs[i], inputs[i])) return fail(MBQC_E_INVALID, "compile_graph: unknown input");
  for (int i = 0; i < d->n_outputs; ++i) {
    if (!index_of(d->outputs[i], outputs[i])) return fail(MBQC_E_INVALID, "compile_graph: unknown output");
    is_output[outputs[i]] = 1;
  }
  // measurements: outputs carry none (else the Python compiler handles them)
  for (int i = 0; i < n; ++i) {
    const int p = d->plane[i];
    if (is_output[i] != (p < 0))
      return fail(MBQC_E_UNSUPPORTED, "compile_graph: measured outputs or unmeasured non-outputs");
    if (p > MBQC_PLANE_Z) return fail(MBQC_E_UNSUPPORTED, "compile_graph: plane %d", p);
    if (d->kind == 0 && p > MBQC_PLANE_Y)
      return fail(MBQC_E_UNSUPPORTED, "compile_graph: only XY planes in the statevector sweep");
  }
  if (d->n_inputs != d->n_outputs)
    return fail(MBQC_E_UNSUPPORTED, "compile_graph: inputs and outputs differ in size (no flow)");

  // flow layers and the measurement order (calculate_order)
  std::vector<int> layer;
  const int fl = flow_layers(g, inputs, outputs, layer);
  if (fl < 0) return fail(MBQC_E_UNSUPPORTED, "compile_graph: flow search depends on set order");
  if (fl == 0) return fail(MBQC_E_UNSUPPORTED, "compile_graph: no causal flow");
  std::vector<int> count(n, 0);
  {
    // count[i] = #{j : layer[i] > layer[j]} via a histogram of layers
    int maxl = 0;
    for (int v : layer) maxl = v > maxl ? v : maxl;
    std::vector<int> below(maxl + 2, 0);
    for (int v : layer) ++below[v + 1];
    for (int l = 1; l <= maxl + 1; ++l) below[l] += below[l - 1];
    for (int i = 0; i < n; ++i) count[i] = below[layer[i]];
  }
  std::vector<int> order;
  order.reserve(n);
  {
    // groups by count descending, graph order inside a group (stable)
    std::vector<std::vector<int>> groups(n + 1);
    for (int i = 0; i < n; ++i) groups[count[i]].push_back(i);
    for (int c = n; c >= 0; --c)
      for (int i : groups[c]) order.push_back(i);
    for (int q = d->n_inputs - 1; q >= 0; --q) {
      const int v = inputs[q];
      for (size_t p = 0; p < order.size(); ++p)
        if (order[p] == v) {
          order.erase(order.begin() + p);
          break;
        }
      order.insert(order.begin(), v);
    }
  }

  // window and the measured nodes (SV: outputs excluded; DM: quantum outputs)
  const int n_in = d->n_inputs;
  int w = d->window_size <= 1 ? n_in + 1 : d->window_size;
  std::vector<int> meas;
  for (int v : order)
    if (!is_output[v]) meas.push_back(v);
  const int M = (int)meas.size();
  // input reorder check (_find_swaps asserts the same elements)
  {
    std::vector<char> seen(n, 0);
    for (int q = 0; q < n_in; ++q) seen[order[q]] = 1;
    for (int q = 0; q < n_in; ++q)
      if (!seen[inputs[q]]) return fail(MBQC_E_UNSUPPORTED, "compile_graph: inputs not first in the order");
  }
  if (n_in > w) return fail(MBQC_E_INVALID, "Input state has %d qubits, but window size is set to %d.", n_in, w);
  if (w > M) return fail(MBQC_E_INVALID, "Window size is set to %d, but schedule only has %d measurements.", w, M);
  if (w > 30) return fail(MBQC_E_UNSUPPORTED, "window size %d exceeds the supported maximum of 30", w);

  for (int p = 0; p < M; ++p)
    if (is_output[order[p]])
      return fail(MBQC_E_UNSUPPORTED, "compile_graph: an output precedes a measured node in the order");
  std::vector<int> pos(n, -1);
  for (int p = 0; p < n; ++p) pos[order[p]] = p;
  t->window = w;
  t->n_nodes = n;
  t->n_steps = M;
  t->n_in = n_in;
  for (int q = 0; q < n_in; ++q) t->in_bits[q] = pos[inputs[q]] % w;
  for (int q = 0; q < 32; ++q) t->init_cz[q] = 0;
  for (int a = 0; a < w; ++a)
    for (int b : g.adj[order[a]])
      if (pos[b] < w && pos[b] > a) t->init_cz[a] |= 1u << pos[b];

  // trainable order: the given labels, else graph order of trainable nodes
  std::vector<int> angle_of(n, -1);
  int A = 0;
  if (d->trainable_order) {
    for (int i = 0; i < d->n_trainable; ++i) {
      int v;
      if (!index_of(d->trainable_order[i], v) || !d->trainable[v])
        return fail(MBQC_E_INVALID, "compile_graph: trainable order names a fixed node");
      angle_of[v] = A++;
    }
  } else {
    for (int i = 0; i < n; ++i)
      if (d->trainable[i]) angle_of[i] = A++;
  }
  t->n_angles = A;
  for (int k = 0; k < M; ++k) {
    const int v = meas[k];
    t->step_plane[k] = d->plane[v];
    t->step_angle[k] = angle_of[v];
    t->step_fixed_angle[k] = angle_of[v] >= 0 ? 0.0 : d->angle[v];
    if (d->trainable[v] && angle_of[v] < 0)
      return fail(MBQC_E_INVALID, "compile_graph: trainable node missing from the trainable order");
    if (k + 1 + w <= n) {
      const int nw = order[k + w];
      uint32_t mask = 0;
      for (int b : g.adj[nw])
        if (pos[b] >= k + 1 && pos[b] < k + w) mask |= 1u << (pos[b] % w);
      t->step_mask[k] = mask;
    } else {
      t->step_mask[k] = kDeadBit;
    }
  }
  // outputs: the qubits left in the window, reordered as the reference does
  std::vector<int> current;
  for (int p = M; p < n && (int)current.size() < w; ++p) current.push_back(order[p]);
  const int n_left = n - M < w ? n - M : w;
  if ((int)current.size() != n_left) return fail(MBQC_E_INVALID, "compile_graph: final window");
  std::vector<int> qout;  // quantum outputs in graph (measurement-dict) order
  for (int i = 0; i < n; ++i)
    if (is_output[i]) qout.push_back(i);
  std::vector<int> fin;
  if (d->kind == 0) {
    fin = (qout != current) ? outputs : current;
  } else {
    fin = (qout != current) ? qout : current;
  }
  if (fin.size() != current.size()) return fail(MBQC_E_INVALID, "compile_graph: output count");
  {
    std::vector<char> inw(n, 0);
    for (int v : current) inw[v] = 1;
    for (int v : fin)
      if (!inw[v]) return fail(MBQC_E_INVALID, "compile_graph: outputs are not the final window");
  }
  t->n_out = (int)fin.size();
  for (size_t j = 0; j < fin.size(); ++j) {
    t->out_bits[j] = pos[fin[j]] % w;
    t->out_nodes[j] = d->nodes[fin[j]];
  }
  for (int p = 0; p < n; ++p) t->schedule[p] = d->nodes[order[p]];
  return MBQC_OK;
}

}  // extern "C"

extern "C" {

int mbqc_plan_create_from_graphs(const mbqc_graph_batch *b, mbqc_plan **plan, int32_t *info) {
  if (!b || b->n_graphs < 0) return fail(MBQC_E_INVALID, "plan_create_from_graphs: bad batch");
  const int G = b->n_graphs;
  if (G == 0) return fail(MBQC_E_INVALID, "plan_create_from_graphs: no graphs");
  if (!b->node_off || !b->edge_off || !b->in_off || !b->out_off || !b->nodes || !b->plane || !b->trainable ||
      !b->angle)
    return fail(MBQC_E_INVALID, "plan_create_from_graphs: null array");
  // per-graph tables, kept alive until the device upload
  struct Tabs {
    std::vector<int32_t> in_bits, step_angle, step_plane, out_bits, out_nodes, schedule;
    std::vector<uint32_t> init_cz, step_mask;
    std::vector<double> step_fixed;
    mbqc_plan_tables t;
  };
  std::vector<Tabs> tabs(G);
  std::vector<mbqc_circuit_desc> descs(G);
  for (int i = 0; i < G; ++i) {
    const int64_t n0 = b->node_off[i], n1 = b->node_off[i + 1];
    const int64_t e0 = b->edge_off[i], e1 = b->edge_off[i + 1];
    const int64_t i0 = b->in_off[i], i1 = b->in_off[i + 1];
    const int64_t o0 = b->out_off[i], o1 = b->out_off[i + 1];
    if (n1 <= n0 || e1 < e0 || i1 < i0 || o1 < o0)
      return fail(MBQC_E_INVALID, "plan_create_from_graphs: graph %d: bad offsets", i);
    mbqc_graph_desc d;
    d.n_nodes = (int32_t)(n1 - n0);
    d.nodes = b->nodes + n0;
    d.n_edges = (int32_t)(e1 - e0);
    d.edges = b->edges ? b->edges + 2 * e0 : nullptr;
    d.n_inputs = (int32_t)(i1 - i0);
    d.inputs = b->inputs ? b->inputs + i0 : nullptr;
    d.n_outputs = (int32_t)(o1 - o0);
    d.outputs = b->outputs ? b->outputs + o0 : nullptr;
    d.plane = b->plane + n0;
    d.trainable = b->trainable + n0;
    d.angle = b->angle + n0;
    d.n_trainable = 0;
    d.trainable_order = nullptr;
    d.window_size = b->window_size;
    d.kind = b->kind;
    Tabs &T = tabs[i];
    const size_t n = (size_t)d.n_nodes;
    T.in_bits.resize(n);
    T.step_angle.resize(n);
    T.step_plane.resize(n);
    T.out_bits.resize(n);
    T.out_nodes.resize(n);
    T.schedule.resize(n);
    T.init_cz.resize(32);
    T.step_mask.resize(n);
    T.step_fixed.resize(n);
    T.t.in_bits = T.in_bits.data();
    T.t.init_cz = T.init_cz.data();
    T.t.step_mask = T.step_mask.data();
    T.t.step_angle = T.step_angle.data();
    T.t.step_plane = T.step_plane.data();
    T.t.step_fixed_angle = T.step_fixed.data();
    T.t.out_bits = T.out_bits.data();
    T.t.out_nodes = T.out_nodes.data();
    T.t.schedule = T.schedule.data();
    const int rc = mbqc_compile_graph(&d, &T.t);
    if (rc != MBQC_OK) {
      const std::string msg = mbqc_last_error();
      return fail(rc, "graph %d: %s", i, msg.c_str());
    }
    mbqc_circuit_desc &c = descs[i];
    c.window = T.t.window;
    c.n_steps = T.t.n_steps;
    c.n_in = T.t.n_in;
    c.n_out = T.t.n_out;
    c.n_angles = T.t.n_angles;
    c.in_bits = T.in_bits.data();
    c.out_bits = T.out_bits.data();
    c.init_cz = T.init_cz.data();
    c.step_mask = T.step_mask.data();
    c.step_angle = T.step_angle.data();
    c.step_plane = T.step_plane.data();
    c.step_fixed_angle = T.step_fixed.data();
    if (info) {
      int32_t *r = info + 5 * (size_t)i;
      r[0] = c.window;
      r[1] = c.n_steps;
      r[2] = c.n_in;
      r[3] = c.n_out;
      r[4] = c.n_angles;
    }
  }
  if (!plan) return MBQC_OK;  // compile only
  return mbqc_plan_create(descs.data(), G, plan);
}

}  // extern "C"
