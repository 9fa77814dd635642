// Tensor-network contraction: the H_eff application of optimal_map
// (operator_map.jl:3-10), the ProjTTN environment updates and the region product
// (extracter.jl:7, :14).
//
// Pairwise contractions are mapped onto (strided-batched) GEMMs without moving data
// whenever the contracted labels form one contiguous axis group of each operand:
//   A = [FA1, K, FA2], B = [K, FB] / [FB, K] / [FB1, K, FB2].
// When FA2 (or FB2) is non-empty the GEMM is batched over it, which is how the
// small operator tensors (W, W1·W2) are applied to a large vector without a
// transpose.  Only when the groups are interleaved, or both operands would need a
// batch, is the smaller operand permuted.  The pairwise order of a network is the
// exact flop-optimal tree (dynamic programming over subsets, the role of
// `contraction_sequence(...; alg="optimal")` at operator_map.jl:7).
#include "nsg_internal.h"

#include <algorithm>
#include <functional>
#include <cmath>
#include <map>
#include <memory>
#include <unordered_map>

namespace nsg {

namespace {

struct LT {
  nsg_tensor* t = nullptr;
  std::vector<int> lab;
  bool conj = false;
  bool owned = false;
};

int64_t prod_dims(const nsg_tensor* t, int b, int e) {
  int64_t p = 1;
  for (int k = b; k < e; ++k) p *= t->dims[k];
  return p;
}

int pos_of(const std::vector<int>& v, int x) {
  for (size_t i = 0; i < v.size(); ++i)
    if (v[i] == x) return int(i);
  return -1;
}

// permute an operand into the label order `order` (conjugating if it carries conj)
LT permute_to(nsg_ctx* c, const LT& a, const std::vector<int>& order, nsg_tensor* into = nullptr) {
  std::vector<int> perm(order.size());
  int64_t dims[NSG_MAX_RANK];
  for (size_t k = 0; k < order.size(); ++k) {
    perm[k] = pos_of(a.lab, order[k]);
    NSG_CHECK(perm[k] >= 0, NSG_ERR_INVALID, "permute_to: label missing");
    dims[k] = a.t->dims[perm[k]];
  }
  LT r;
  r.t = into ? into : new_tensor(c, a.t->dtype, int(order.size()), dims, false);
  r.lab = order;
  r.owned = (into == nullptr);
  permute(c, a.t, perm.data(), a.conj, r.t);
  return r;
}

void release(nsg_ctx* c, LT& a) {
  if (a.owned) free_tensor(c, a.t);
  a.t = nullptr;
  a.owned = false;
}

// Where the contracted labels sit inside an operand: [F1, K, F2] with K contiguous.
struct Layout {
  bool contiguous = false;
  int s = 0;                 // first K position
  std::vector<int> korder;   // K labels in stored order
};

Layout classify(const LT& a, const std::vector<int>& K) {
  Layout L;
  std::vector<int> pos;
  for (int k : K) pos.push_back(pos_of(a.lab, k));
  std::sort(pos.begin(), pos.end());
  if (K.empty()) {
    L.contiguous = true;
    L.s = int(a.lab.size());
    return L;
  }
  L.contiguous = (pos.back() - pos.front() + 1 == int(pos.size()));
  L.s = pos.front();
  for (int p : pos) L.korder.push_back(a.lab[p]);
  return L;
}

int with_conj(int op, bool conj) {
  if (!conj) return op;
  return op == OP_N ? OP_R : (op == OP_T ? OP_C : op);
}

}  // namespace

// Contract two labeled tensors over their shared labels.  `final_order`, when
// given, is the requested label order of the result; `into`, when given, receives
// the result (its shape must match).
static LT contract_pair(nsg_ctx* c, LT A, LT B, const std::vector<int>* final_order, nsg_tensor* into) {
  NSG_CHECK(A.t->dtype == B.t->dtype, NSG_ERR_INVALID, "contract: dtype mismatch");
  const int dtype = A.t->dtype;
  std::vector<int> K;
  for (int l : A.lab)
    if (pos_of(B.lab, l) >= 0) K.push_back(l);
  auto dim_of = [&](int l) -> int64_t {
    int p = pos_of(A.lab, l);
    if (p >= 0) return A.t->dims[p];
    return B.t->dims[pos_of(B.lab, l)];
  };
  for (int l : K)
    NSG_CHECK(A.t->dims[pos_of(A.lab, l)] == B.t->dims[pos_of(B.lab, l)], NSG_ERR_INVALID,
              "contract: dimension mismatch on a shared label");
  std::vector<LT> temps;
  Layout la = classify(A, K), lb = classify(B, K);
  int ra = int(A.lab.size()), rb = int(B.lab.size());
  int nk = int(K.size());
  auto batched = [&](const Layout& L, int r) { return L.contiguous && L.s > 0 && L.s + nk < r; };
  // Fix operands that cannot be used in place.
  auto canon_A = [&](const std::vector<int>& korder) {
    std::vector<int> ord;
    for (int l : A.lab)
      if (pos_of(K, l) < 0) ord.push_back(l);
    for (int l : korder) ord.push_back(l);
    LT P = permute_to(c, A, ord);
    temps.push_back(P);
    A = P;
    A.owned = false;
    la = classify(A, K);
  };
  auto canon_B = [&](const std::vector<int>& korder) {
    std::vector<int> ord(korder.begin(), korder.end());
    for (int l : B.lab)
      if (pos_of(K, l) < 0) ord.push_back(l);
    LT P = permute_to(c, B, ord);
    temps.push_back(P);
    B = P;
    B.owned = false;
    lb = classify(B, K);
  };
  if (!la.contiguous && !lb.contiguous) {
    canon_A(K);
    canon_B(la.korder);
  } else if (!la.contiguous) {
    canon_A(lb.korder);
  } else if (!lb.contiguous) {
    canon_B(la.korder);
  }
  if (batched(la, ra) && batched(lb, rb)) {
    if (A.t->size <= B.t->size)
      canon_A(lb.korder);
    else
      canon_B(la.korder);
  }
  if (la.korder != lb.korder) {
    // permute the smaller operand to the other's K order (unless that one is batched)
    bool permA = A.t->size <= B.t->size;
    if (batched(lb, rb)) permA = true;
    if (batched(la, ra)) permA = false;
    if (permA)
      canon_A(lb.korder);
    else
      canon_B(la.korder);
  }
  NSG_CHECK(la.contiguous && lb.contiguous && la.korder == lb.korder, NSG_ERR_INVALID,
            "contract: internal layout error");
  ra = int(A.lab.size());
  rb = int(B.lab.size());
  int64_t Kd = 1;
  for (int l : K) Kd *= dim_of(l);
  std::vector<int> FA1(A.lab.begin(), A.lab.begin() + la.s), FA2(A.lab.begin() + la.s + nk, A.lab.end());
  std::vector<int> FB1(B.lab.begin(), B.lab.begin() + lb.s), FB2(B.lab.begin() + lb.s + nk, B.lab.end());
  int64_t a1 = prod_dims(A.t, 0, la.s), a2 = prod_dims(A.t, la.s + nk, ra);
  int64_t b1 = prod_dims(B.t, 0, lb.s), b2 = prod_dims(B.t, lb.s + nk, rb);

  GemmArgs g;
  g.dtype = dtype;
  g.K = Kd;
  std::vector<int> outlab;
  bool transposed = false;
  if (!FA1.empty() && !FA2.empty()) {
    // A batched over FA2: C_b[FA1, FB] = A_b[FA1, K] op(B)
    int opB;
    int64_t ldb;
    std::vector<int> FB;
    if (FB1.empty()) {
      opB = OP_N;
      ldb = Kd;
      FB = FB2;
    } else {
      opB = OP_T;
      ldb = b1;
      FB = FB1;
    }
    int64_t nb = FB1.empty() ? b2 : b1;
    g.M = a1;
    g.N = nb;
    g.A = A.t->data;
    g.lda = a1;
    g.strideA = a1 * Kd;
    g.opA = with_conj(OP_N, A.conj);
    g.B = B.t->data;
    g.ldb = ldb;
    g.strideB = 0;
    g.opB = with_conj(opB, B.conj);
    g.ldc = a1;
    g.strideC = a1 * nb;
    g.batch = a2;
    outlab = FA1;
    outlab.insert(outlab.end(), FB.begin(), FB.end());
    outlab.insert(outlab.end(), FA2.begin(), FA2.end());
  } else if (!FB1.empty() && !FB2.empty()) {
    // B batched over FB2: C_b[FA, FB1] = op(A) B_b[FB1, K]^T
    int opA;
    int64_t lda;
    std::vector<int> FA;
    if (FA2.empty()) {
      opA = OP_N;
      lda = a1;
      FA = FA1;
    } else {
      opA = OP_T;
      lda = Kd;
      FA = FA2;
    }
    int64_t ma = FA2.empty() ? a1 : a2;
    g.M = ma;
    g.N = b1;
    g.A = A.t->data;
    g.lda = lda;
    g.strideA = 0;
    g.opA = with_conj(opA, A.conj);
    g.B = B.t->data;
    g.ldb = b1;
    g.strideB = b1 * Kd;
    g.opB = with_conj(OP_T, B.conj);
    g.ldc = ma;
    g.strideC = ma * b1;
    g.batch = b2;
    outlab = FA;
    outlab.insert(outlab.end(), FB1.begin(), FB1.end());
    outlab.insert(outlab.end(), FB2.begin(), FB2.end());
  } else {
    // plain GEMM
    std::vector<int> FA = FA2.empty() ? FA1 : FA2;
    std::vector<int> FB = FB1.empty() ? FB2 : FB1;
    int64_t M = FA2.empty() ? a1 : a2;
    int64_t N = FB1.empty() ? b2 : b1;
    int opA = FA2.empty() ? OP_N : OP_T;  // stored [FA, K] -> N ; [K, FA] -> T
    int64_t lda = FA2.empty() ? M : Kd;
    int opB = FB1.empty() ? OP_N : OP_T;  // stored [K, FB] -> N ; [FB, K] -> T
    int64_t ldb = FB1.empty() ? Kd : N;
    std::vector<int> natural = FA;
    natural.insert(natural.end(), FB.begin(), FB.end());
    std::vector<int> swapped = FB;
    swapped.insert(swapped.end(), FA.begin(), FA.end());
    transposed = final_order && *final_order != natural && *final_order == swapped;
    g.batch = 1;
    g.strideA = g.strideB = g.strideC = 0;
    if (!transposed) {
      g.M = M;
      g.N = N;
      g.A = A.t->data;
      g.lda = lda;
      g.opA = with_conj(opA, A.conj);
      g.B = B.t->data;
      g.ldb = ldb;
      g.opB = with_conj(opB, B.conj);
      g.ldc = M;
      outlab = natural;
    } else {
      // C^T = op(B)^T op(A)^T
      auto tr = [](int op) { return op == OP_N ? OP_T : (op == OP_T ? OP_N : (op == OP_C ? OP_R : OP_C)); };
      g.M = N;
      g.N = M;
      g.A = B.t->data;
      g.lda = ldb;
      g.opA = tr(with_conj(opB, B.conj));
      g.B = A.t->data;
      g.ldb = lda;
      g.opB = tr(with_conj(opA, A.conj));
      g.ldc = N;
      outlab = swapped;
    }
  }
  int64_t odims[NSG_MAX_RANK];
  NSG_CHECK(outlab.size() <= NSG_MAX_RANK, NSG_ERR_UNSUPPORTED, "contract: result rank above 16");
  for (size_t k = 0; k < outlab.size(); ++k) odims[k] = dim_of(outlab[k]);
  bool need_final_perm = final_order && *final_order != outlab;
  LT R;
  R.lab = outlab;
  if (into && !need_final_perm) {
    NSG_CHECK(into->size == [&] { int64_t p = 1; for (size_t k = 0; k < outlab.size(); ++k) p *= odims[k]; return p; }(),
              NSG_ERR_INVALID, "contract: output tensor has the wrong size");
    R.t = into;
    R.owned = false;
  } else {
    R.t = new_tensor(c, dtype, int(outlab.size()), odims, false);
    R.owned = true;
  }
  g.C = R.t->data;
  gemm(c, g);
  c->contractions += 1;
  for (auto& t : temps) release(c, t);
  if (need_final_perm) {
    LT P = permute_to(c, R, *final_order, into);
    release(c, R);
    return P;
  }
  return R;
}

// ---------------------------------------------------------------------------
// contraction trees
// ---------------------------------------------------------------------------
struct Node {
  int leaf = -1;          // tensor index for leaves
  int left = -1, right = -1;
  uint32_t mask = 0;
  std::vector<int> open;  // labels of the intermediate
  double flops = 0;       // MACs of this step
};

struct Tree {
  std::vector<Node> nodes;
  int root = -1;
  double total_macs = 0;
};

static Tree optimal_tree(const std::vector<std::vector<int>>& labs, const std::vector<int>& out_labels,
                         const std::unordered_map<int, int64_t>& dims) {
  int n = int(labs.size());
  NSG_CHECK(n >= 1 && n <= 12, NSG_ERR_UNSUPPORTED, "contract: 1..12 tensors");
  uint32_t full = (n == 32) ? 0xffffffffu : ((1u << n) - 1);
  // label -> mask of tensors containing it
  std::map<int, uint32_t> where;
  for (int i = 0; i < n; ++i)
    for (int l : labs[i]) where[l] |= (1u << i);
  std::map<int, bool> in_out;
  for (int l : out_labels) in_out[l] = true;
  auto open_of = [&](uint32_t S) {
    std::vector<int> o;
    for (auto& [l, m] : where) {
      bool inside = (m & S) != 0;
      bool outside = (m & ~S & full) != 0 || in_out.count(l);
      if (inside && outside) o.push_back(l);
    }
    return o;
  };
  auto size_of = [&](const std::vector<int>& ls) {
    double p = 1;
    for (int l : ls) p *= double(dims.at(l));
    return p;
  };
  std::vector<double> cost(size_t(1) << n, 0.0);
  std::vector<uint32_t> split(size_t(1) << n, 0);
  std::vector<std::vector<int>> openS(size_t(1) << n);
  for (uint32_t S = 1; S <= full; ++S) openS[S] = open_of(S);
  for (uint32_t S = 1; S <= full; ++S) {
    if ((S & (S - 1)) == 0) continue;  // leaf
    double best = INFINITY;
    uint32_t bs = 0;
    for (uint32_t S1 = (S - 1) & S; S1 > 0; S1 = (S1 - 1) & S) {
      uint32_t S2 = S & ~S1;
      if (S1 < S2) continue;
      // labels involved in the step = open(S1) ∪ open(S2)
      std::vector<int> inv = openS[S1];
      for (int l : openS[S2])
        if (pos_of(inv, l) < 0) inv.push_back(l);
      double f = cost[S1] + cost[S2] + size_of(inv);
      if (f < best) {
        best = f;
        bs = S1;
      }
    }
    cost[S] = best;
    split[S] = bs;
  }
  Tree T;
  std::function<int(uint32_t)> build = [&](uint32_t S) -> int {
    Node nd;
    nd.mask = S;
    nd.open = openS[S];
    if ((S & (S - 1)) == 0) {
      int i = 0;
      while (!((S >> i) & 1)) ++i;
      nd.leaf = i;
      nd.open = labs[i];
    } else {
      uint32_t S1 = split[S], S2 = S & ~S1;
      nd.left = build(S1);
      nd.right = build(S2);
      std::vector<int> inv = T.nodes[nd.left].open;
      for (int l : T.nodes[nd.right].open)
        if (pos_of(inv, l) < 0) inv.push_back(l);
      nd.flops = size_of(inv);
      T.total_macs += nd.flops;
    }
    T.nodes.push_back(nd);
    return int(T.nodes.size()) - 1;
  };
  T.root = build(full);
  return T;
}

}  // namespace nsg

using namespace nsg;

struct nsg_linmap {
  int n_fixed = 0;
  std::vector<nsg_tensor*> fixed;            // borrowed
  std::vector<std::vector<int>> labs;        // fixed..., x
  std::vector<int> conj;
  std::vector<int> x_labels, y_labels;
  Tree tree;
  std::map<int, LT> cached;                  // node index -> precomputed fixed-only result
  int dtype = NSG_F64;
  double flops = 0;
};

namespace nsg {

static LT eval_node(nsg_ctx* c, nsg_linmap* m, int ni, const LT& xleaf, const std::vector<int>* final_order,
                    nsg_tensor* into) {
  Node& nd = m->tree.nodes[ni];
  auto it = m->cached.find(ni);
  if (it != m->cached.end()) {
    LT r = it->second;
    r.owned = false;
    return r;
  }
  if (nd.leaf >= 0) {
    if (nd.leaf == m->n_fixed) return xleaf;
    LT r;
    r.t = m->fixed[nd.leaf];
    r.lab = m->labs[nd.leaf];
    r.conj = m->conj[nd.leaf] != 0;
    r.owned = false;
    return r;
  }
  LT a = eval_node(c, m, nd.left, xleaf, nullptr, nullptr);
  LT b = eval_node(c, m, nd.right, xleaf, nullptr, nullptr);
  LT r = contract_pair(c, a, b, final_order, into);
  release(c, a);
  release(c, b);
  return r;
}

}  // namespace nsg

extern "C" {

int nsg_contract(nsg_ctx* c, int n, nsg_tensor* const* tensors, const int32_t* labels, const int* conj,
                 int out_rank, const int32_t* out_labels, nsg_tensor** out) {
  NSG_API_BEGIN(c)
  NSG_CHECK(c && tensors && labels && out && n >= 1, NSG_ERR_INVALID, "null argument");
  std::vector<std::vector<int>> labs(n);
  std::unordered_map<int, int64_t> dims;
  std::map<int, int> count;
  int off = 0;
  int dtype = tensors[0]->dtype;
  for (int i = 0; i < n; ++i) {
    NSG_CHECK(tensors[i] && tensors[i]->dtype == dtype, NSG_ERR_INVALID, "contract: null tensor or mixed dtypes");
    for (int k = 0; k < tensors[i]->rank; ++k) {
      int l = labels[off + k];
      labs[i].push_back(l);
      auto d = dims.find(l);
      NSG_CHECK(d == dims.end() || d->second == tensors[i]->dims[k], NSG_ERR_INVALID,
                "contract: label " + std::to_string(l) + " has two different dimensions");
      dims[l] = tensors[i]->dims[k];
      count[l]++;
    }
    off += tensors[i]->rank;
  }
  std::vector<int> outl(out_labels, out_labels + out_rank);
  for (int l : outl) NSG_CHECK(count[l] == 1, NSG_ERR_INVALID, "contract: output label must appear exactly once");
  for (auto& [l, k] : count) {
    NSG_CHECK(k <= 2, NSG_ERR_UNSUPPORTED, "contract: a label appears in more than two tensors");
    if (k == 1) NSG_CHECK(pos_of(outl, l) >= 0, NSG_ERR_INVALID, "contract: unmatched label missing from output");
  }
  if (n == 1) {
    LT a;
    a.t = tensors[0];
    a.lab = labs[0];
    a.conj = conj && conj[0];
    LT r = permute_to(c, a, outl);
    *out = r.t;
  } else {
    nsg_linmap m;
    m.n_fixed = n - 1;
    m.fixed.assign(tensors, tensors + n - 1);
    m.labs = labs;
    for (int i = 0; i < n; ++i) m.conj.push_back(conj ? conj[i] : 0);
    m.tree = optimal_tree(labs, outl, dims);
    LT x;
    x.t = tensors[n - 1];
    x.lab = labs[n - 1];
    x.conj = m.conj[n - 1] != 0;
    LT r = eval_node(c, &m, m.tree.root, x, &outl, nullptr);
    if (!r.owned) {  // the root was a leaf (cannot happen for n >= 2) -> copy
      LT p = permute_to(c, r, outl);
      r = p;
    }
    *out = r.t;
  }
  NSG_API_END(c)
}

int nsg_linmap_create(nsg_ctx* c, int n_fixed, nsg_tensor* const* fixed, const int32_t* labels, const int* conj,
                      int x_rank, const int32_t* x_labels, const int32_t* y_labels, nsg_linmap** out) {
  NSG_API_BEGIN(c)
  NSG_CHECK(c && out && x_labels && y_labels && n_fixed >= 0, NSG_ERR_INVALID, "null argument");
  auto* m = new nsg_linmap();
  std::unique_ptr<nsg_linmap> guard(m);
  m->n_fixed = n_fixed;
  m->fixed.assign(fixed, fixed + n_fixed);
  std::unordered_map<int, int64_t> dims;
  int off = 0;
  for (int i = 0; i < n_fixed; ++i) {
    std::vector<int> l(labels + off, labels + off + fixed[i]->rank);
    for (int k = 0; k < fixed[i]->rank; ++k) {
      auto d = dims.find(l[k]);
      NSG_CHECK(d == dims.end() || d->second == fixed[i]->dims[k], NSG_ERR_INVALID,
                "linmap: label with two different dimensions");
      dims[l[k]] = fixed[i]->dims[k];
    }
    off += fixed[i]->rank;
    m->labs.push_back(l);
    m->conj.push_back(conj ? conj[i] : 0);
    if (i == 0) m->dtype = fixed[i]->dtype;
    NSG_CHECK(fixed[i]->dtype == m->dtype, NSG_ERR_INVALID, "linmap: mixed dtypes");
  }
  m->x_labels.assign(x_labels, x_labels + x_rank);
  m->y_labels.assign(y_labels, y_labels + x_rank);
  // x's dims are inferred from the y labels' dimensions in the fixed tensors where possible;
  // x labels must be matched by fixed tensors or pass straight through to y.
  m->labs.push_back(m->x_labels);
  m->conj.push_back(0);
  for (size_t k = 0; k < m->x_labels.size(); ++k) {
    int xl = m->x_labels[k], yl = m->y_labels[k];
    int64_t d = -1;
    if (dims.count(xl)) d = dims[xl];
    if (dims.count(yl)) {
      NSG_CHECK(d < 0 || d == dims[yl], NSG_ERR_INVALID, "linmap: x and y label dimensions differ");
      d = dims[yl];
    }
    NSG_CHECK(d > 0, NSG_ERR_INVALID, "linmap: x label not connected to the fixed tensors");
    dims[xl] = d;
    if (!dims.count(yl)) dims[yl] = d;
  }
  m->tree = optimal_tree(m->labs, m->y_labels, dims);
  m->flops = m->tree.total_macs * (m->dtype == NSG_C128 ? 8.0 : 2.0);
  // precompute fixed-only subtrees (largest ones only: a node whose parent contains x)
  uint32_t xbit = 1u << n_fixed;
  for (size_t ni = 0; ni < m->tree.nodes.size(); ++ni) {
    Node& nd = m->tree.nodes[ni];
    if (nd.leaf >= 0 || (nd.mask & xbit)) continue;
    // is the parent an x-containing node?
    bool parent_has_x = false;
    for (auto& p : m->tree.nodes)
      if ((p.left == int(ni) || p.right == int(ni)) && (p.mask & xbit)) parent_has_x = true;
    if (!parent_has_x) continue;
    LT dummy;
    LT r = eval_node(c, m, int(ni), dummy, nullptr, nullptr);
    m->cached[int(ni)] = r;
  }
  *out = guard.release();
  NSG_API_END(c)
}

int nsg_linmap_apply(nsg_ctx* c, nsg_linmap* m, const nsg_tensor* x, nsg_tensor* y) {
  NSG_API_BEGIN(c)
  NSG_CHECK(c && m && x && y, NSG_ERR_INVALID, "null argument");
  NSG_CHECK(x->rank == int(m->x_labels.size()) && y->size == x->size && x->dtype == y->dtype &&
                (m->n_fixed == 0 || x->dtype == m->dtype),
            NSG_ERR_INVALID, "linmap_apply: x/y shape or dtype mismatch");
  PhaseScope phase(c, NSG_PHASE_HEFF);
  LT xl;
  xl.t = const_cast<nsg_tensor*>(x);
  xl.lab = m->x_labels;
  if (m->n_fixed == 0) {
    NSG_CUDA(cudaMemcpyAsync(y->data, x->data, x->bytes, cudaMemcpyDeviceToDevice, c->stream));
  } else {
    LT r = eval_node(c, m, m->tree.root, xl, &m->y_labels, y);
    if (r.t != y) {
      NSG_CUDA(cudaMemcpyAsync(y->data, r.t->data, y->bytes, cudaMemcpyDeviceToDevice, c->stream));
      release(c, r);
    }
  }
  c->applies += 1;
  NSG_API_END(c)
}

int nsg_linmap_release(nsg_ctx* c, nsg_linmap* m) {
  NSG_API_BEGIN(c)
  if (m) {
    for (auto& [k, v] : m->cached) {
      LT t = v;
      t.owned = true;
      release(c, t);
    }
    delete m;
  }
  NSG_API_END(c)
}

int nsg_linmap_flops(const nsg_linmap* m, double* flops) {
  if (!m || !flops) return NSG_ERR_INVALID;
  *flops = m->flops;
  return NSG_OK;
}

}  // extern "C"

// internal entry for other translation units
namespace nsg {
void linmap_apply(nsg_ctx* c, nsg_linmap* m, const nsg_tensor* x, nsg_tensor* y) {
  int rc = nsg_linmap_apply(c, m, x, y);
  if (rc != NSG_OK) throw Error(rc, c->err);
}
}  // namespace nsg
