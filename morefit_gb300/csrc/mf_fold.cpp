// Folding of linearly dependent input columns of a REDUCE kernel.
//
// MoreFit's fitter hoists every event-only factor of the density into its own
// column (reference include/fitter.hh:345-375), one column per term of the
// PDF. The K*mumu P-wave density (include/physicspdfs.hh:39-77) has 11 such
// terms, and in the printed kernels (include/fitter.hh:612-657) the density is
// a linear form of those columns whose coefficients are parameter-only
// expressions: S9*b3 + S8*b4 + ... - Fl*b10 + pb0*b11 + pb0*b12 + Fl*b13.
// Coefficients that are equal or opposite for every parameter value (pb0 for
// b11 and b12, -Fl and Fl for b10 and b13) mean that the kernel only ever
// needs their combinations, b11 + b12 and b10 - b13: 9 columns instead of 11.
//
// The pass finds every linear form of input columns with parameter-only
// coefficients in the DAG (its "linear roots"), samples the coefficients at
// random parameter values, and takes the column rank of those samples by
// Gram-Schmidt in column order. Columns that are combinations of earlier
// (pivot) columns are folded into them once per dataset:
//   y_m = x_{p_m} + sum_d M[d][m] x_d
// and every linear root is rewritten as sum_m c_{p_m}(params) * y_m, where
// c_{p_m} is the root's own coefficient of the pivot column. The relations are
// verified on a second, independent set of samples; any doubt (a conditional
// or non-finite coefficient, a failed check) leaves the kernel unfolded.
#include <cmath>
#include <cstdint>
#include <map>
#include <memory>
#include <stdexcept>
#include <vector>

#include "mf_lower.h"

namespace mf {

namespace {

enum class K : uint8_t { Dead, Uniform, Affine, Other };

struct Affine {
  std::map<int, int> coef;  // input column -> coefficient node (new DAG)
  int cst = -1;             // parameter-only constant term (new DAG), -1 = none
};

// Copies a parameter-only node of `src` into `dst`.
int copy_uniform(const std::vector<Node>& ns, int id, Dag& dst, std::vector<int>& memo) {
  if (memo[id] >= 0) return memo[id];
  const Node& n = ns[id];
  int r = -1;
  switch (n.op) {
    case Op::Const: r = dst.constant(n.value); break;
    case Op::Param: r = dst.unary(Op::Param, n.index); break;
    case Op::Input: throw std::runtime_error("fold: input in a parameter-only node");
    case Op::Add: case Op::Sub: case Op::Mul: case Op::Div: case Op::Pow:
      r = dst.binary(n.op, copy_uniform(ns, n.a, dst, memo), copy_uniform(ns, n.b, dst, memo));
      break;
    case Op::Cmp: r = dst.compare(n.cmp, copy_uniform(ns, n.a, dst, memo), copy_uniform(ns, n.b, dst, memo)); break;
    case Op::Select:
      r = dst.select(copy_uniform(ns, n.a, dst, memo), copy_uniform(ns, n.b, dst, memo),
                     copy_uniform(ns, n.c, dst, memo));
      break;
    default: r = dst.unary(n.op, copy_uniform(ns, n.a, dst, memo)); break;
  }
  memo[id] = r;
  return r;
}

bool has_conditional(const std::vector<Node>& ns, int id, std::vector<char>& seen) {
  if (id < 0 || seen[id]) return false;
  seen[id] = 1;
  const Node& n = ns[id];
  if (n.op == Op::Cmp || n.op == Op::Select) return true;
  if (n.op == Op::Const || n.op == Op::Param || n.op == Op::Input) return false;
  return has_conditional(ns, n.a, seen) || has_conditional(ns, n.b, seen) || has_conditional(ns, n.c, seen);
}

// Deterministic parameter samples: magnitudes in [0.5, 2), random signs.
std::vector<std::vector<double>> samples(size_t count, size_t np, uint64_t seed) {
  uint64_t s = seed;
  auto next = [&s]() {
    s += 0x9e3779b97f4a7c15ULL;
    uint64_t z = s;
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
    return z ^ (z >> 31);
  };
  std::vector<std::vector<double>> out(count, std::vector<double>(np));
  for (auto& v : out)
    for (auto& x : v) {
      const uint64_t r = next();
      const double u = double(r >> 11) * 0x1.0p-53;
      x = (r & 1) ? -(0.5 + 1.5 * u) : (0.5 + 1.5 * u);
    }
  return out;
}

// A small rational p/q (q <= 64) within 1e-13 of v, or v itself.
double snap(double v) {
  for (int q = 1; q <= 64; q++) {
    const double p = std::nearbyint(v * q);
    if (std::fabs(v - p / q) <= 1e-13 * std::max(1.0, std::fabs(v))) return p / q;
  }
  return v;
}

// Linear relations among the source columns that every linear root's
// coefficients satisfy: pivots (independent columns, in column order),
// dependents, and M[d][m] with coef_d = sum_m M[d][m] coef_{pivot m}.
// False when there are none or anything is doubtful.
bool find_relations(const Dag& d2, const std::vector<Affine>& aff, const std::vector<int>& lroots,
                    const std::map<int, int>& colpos, size_t np, const std::vector<std::string>& param_defs,
                    std::vector<int>& pivots, std::vector<int>& dependents, std::vector<std::vector<double>>& M) {
  const int J = int(colpos.size());
  {
    const auto& n2 = d2.nodes();
    std::vector<char> seen(n2.size(), 0);
    for (int r : lroots)
      for (auto& [col, c] : aff[r].coef)
        if (has_conditional(n2, c, seen)) return false;
  }
  // Parameters defined by expressions of the others take their defined value
  // in every sample (definitions in parameter order; a definition may use
  // parameters defined before it).
  Dag defs({}, d2.param_names());
  std::vector<std::pair<int, int>> def_roots;  // (parameter index, root)
  for (size_t i = 0; i < param_defs.size() && i < np; i++)
    if (!param_defs[i].empty()) def_roots.push_back({int(i), defs.parse(param_defs[i])});
  auto sample_set = [&](size_t count, uint64_t seed) {
    auto S = samples(count, np, seed);
    for (auto& pv : S)
      for (auto& [i, r] : def_roots) pv[i] = defs.eval(r, {}, pv);
    return S;
  };
  // Sample matrix: one row per (sample, linear root), one column per source column.
  auto matrix = [&](uint64_t seed, size_t count, std::vector<std::vector<double>>& Z) {
    Z.assign(J, {});
    for (const auto& pv : sample_set(count, seed))
      for (int r : lroots) {
        std::vector<double> row(J, 0.0);
        for (auto& [col, c] : aff[r].coef) {
          const double v = d2.eval(c, {}, pv);
          if (!std::isfinite(v)) return false;
          row[colpos.at(col)] = v;
        }
        for (int j = 0; j < J; j++) Z[j].push_back(row[j]);
      }
    return true;
  };
  std::vector<std::vector<double>> Z, Zv;
  if (!matrix(0x6d6f726566697431ULL, size_t(J) + 6, Z)) return false;
  if (!matrix(0x6d6f726566697432ULL, size_t(J) + 6, Zv)) return false;
  const size_t R = Z[0].size();
  auto dot = [R](const std::vector<double>& a, const std::vector<double>& b) {
    double s = 0.0;
    for (size_t k = 0; k < R; k++) s += a[k] * b[k];
    return s;
  };

  // Modified Gram-Schmidt in column order: Q (orthonormal), Rm (upper triangular).
  std::vector<std::vector<double>> Q;
  std::vector<std::vector<double>> coefs(J);  // coefficients of column j in the Q basis
  for (int j = 0; j < J; j++) {
    const double norm0 = std::sqrt(dot(Z[j], Z[j]));
    std::vector<double> v = Z[j];
    std::vector<double> c(Q.size(), 0.0);
    for (size_t q = 0; q < Q.size(); q++) {
      c[q] = dot(Q[q], v);
      for (size_t k = 0; k < R; k++) v[k] -= c[q] * Q[q][k];
    }
    const double rn = std::sqrt(dot(v, v));
    if (norm0 > 0.0 && rn <= 1e-9 * norm0) {
      dependents.push_back(j);
      coefs[j] = c;
      continue;
    }
    if (norm0 == 0.0) {  // a column whose coefficients vanish everywhere: drop
      dependents.push_back(j);
      coefs[j] = c;
      continue;
    }
    for (auto& x : v) x /= rn;
    Q.push_back(v);
    c.push_back(rn);
    coefs[j] = c;
    pivots.push_back(j);
  }
  if (dependents.empty()) return false;
  const int r = int(pivots.size());
  // Rm[q][m] = coefficient of pivot m's column on Q[q]; solve Rm * x = c for each dependent.
  for (auto& row : M) row.assign(r, 0.0);
  for (int d : dependents) {
    std::vector<double> c = coefs[d];
    c.resize(size_t(r), 0.0);
    std::vector<double> x(r, 0.0);
    for (int m = r - 1; m >= 0; m--) {
      double s = c[m];
      // upper-triangular entry (m, t) is coefs[pivots[t]][m]
      for (int t = m + 1; t < r; t++) s -= coefs[pivots[t]][m] * x[t];
      x[m] = s / coefs[pivots[m]][m];
    }
    for (int m = 0; m < r; m++) M[d][m] = snap(x[m]);
  }
  // Verify every relation on the independent samples.
  for (int d : dependents) {
    for (size_t k = 0; k < Zv[d].size(); k++) {
      double s = 0.0, mag = std::fabs(Zv[d][k]);
      for (int m = 0; m < r; m++) {
        s += M[d][m] * Zv[pivots[m]][k];
        mag += std::fabs(M[d][m] * Zv[pivots[m]][k]);
      }
      if (std::fabs(Zv[d][k] - s) > 1e-11 * mag + 1e-300) return false;
    }
  }

  return true;
}

}  // namespace

FoldResult fold_columns(const Dag& dag, const std::vector<int>& roots, const std::vector<std::string>& param_defs) {
  FoldResult res;
  const auto& ns = dag.nodes();
  const size_t N = ns.size();
  std::vector<char> live(N, 0);
  {
    std::vector<int> st(roots.begin(), roots.end());
    while (!st.empty()) {
      const int id = st.back();
      st.pop_back();
      if (id < 0 || live[id]) continue;
      live[id] = 1;
      const Node& n = ns[id];
      if (n.op == Op::Input || n.op == Op::Param || n.op == Op::Const) continue;
      st.push_back(n.a);
      st.push_back(n.b);
      st.push_back(n.c);
    }
  }
  // The rewritten DAG: its input indices are the prepared columns.
  auto work = std::make_unique<Dag>(dag.input_names(), dag.param_names());
  Dag& d2 = *work;
  std::vector<int> umemo(N, -1);
  std::vector<K> kind(N, K::Dead);
  std::vector<Affine> aff(N);
  const int one = d2.constant(1.0);

  // Node ids are topological (children are interned before their parents).
  for (size_t i = 0; i < N; i++) {
    if (!live[i]) continue;
    const Node& n = ns[i];
    if (n.uniform) {
      kind[i] = K::Uniform;
      continue;
    }
    if (n.op == Op::Input) {
      kind[i] = K::Affine;
      aff[i].coef[n.index] = one;
      continue;
    }
    // A linear form with a parameter-only constant term (x - mu) is kept
    // as it is written: distributing a factor over it, or merging it into a
    // larger form, would round mu*f (or mu + nu) once for all events, a
    // systematic error where the written form rounds per event.
    auto lin = [&](int c) {
      return c >= 0 && (kind[c] == K::Uniform || (kind[c] == K::Affine && aff[c].cst < 0));
    };
    auto as_aff = [&](int c) {
      if (kind[c] == K::Affine) return aff[c];
      Affine a;
      a.cst = copy_uniform(ns, c, d2, umemo);
      return a;
    };
    if ((n.op == Op::Add || n.op == Op::Sub) && lin(n.a) && lin(n.b)) {
      Affine a = as_aff(n.a), b = as_aff(n.b);
      const bool sub = n.op == Op::Sub;
      for (auto& [col, cb] : b.coef) {
        auto it = a.coef.find(col);
        if (it == a.coef.end())
          a.coef[col] = sub ? d2.unary(Op::Neg, cb) : cb;
        else
          it->second = d2.binary(sub ? Op::Sub : Op::Add, it->second, cb);
      }
      if (b.cst >= 0)
        a.cst = a.cst < 0 ? (sub ? d2.unary(Op::Neg, b.cst) : b.cst) : d2.binary(sub ? Op::Sub : Op::Add, a.cst, b.cst);
      kind[i] = K::Affine;
      aff[i] = std::move(a);
      continue;
    }
    if (n.op == Op::Neg && (lin(n.a) || kind[n.a] == K::Affine)) {  // exact
      Affine a = as_aff(n.a);
      for (auto& [col, c] : a.coef) c = d2.unary(Op::Neg, c);
      if (a.cst >= 0) a.cst = d2.unary(Op::Neg, a.cst);
      kind[i] = K::Affine;
      aff[i] = std::move(a);
      continue;
    }
    if (n.op == Op::Mul && ((kind[n.a] == K::Uniform && kind[n.b] == K::Affine && lin(n.b)) ||
                            (kind[n.a] == K::Affine && kind[n.b] == K::Uniform && lin(n.a)))) {
      const bool left_u = kind[n.a] == K::Uniform;
      const int u = copy_uniform(ns, left_u ? n.a : n.b, d2, umemo);
      Affine a = aff[left_u ? n.b : n.a];
      for (auto& [col, c] : a.coef) c = left_u ? d2.binary(Op::Mul, u, c) : d2.binary(Op::Mul, c, u);
      if (a.cst >= 0) a.cst = left_u ? d2.binary(Op::Mul, u, a.cst) : d2.binary(Op::Mul, a.cst, u);
      kind[i] = K::Affine;
      aff[i] = std::move(a);
      continue;
    }
    kind[i] = K::Other;
  }

  // Linear roots: affine nodes used by a non-affine node or returned.
  std::vector<char> is_root(N, 0);
  for (size_t i = 0; i < N; i++) {
    if (kind[i] != K::Other) continue;
    for (int c : {ns[i].a, ns[i].b, ns[i].c})
      if (c >= 0 && kind[c] == K::Affine) is_root[c] = 1;
  }
  for (int r : roots)
    if (kind[r] == K::Affine) is_root[r] = 1;
  std::vector<int> lroots;
  std::map<int, int> colpos;  // source column -> position in the sample matrix
  for (size_t i = 0; i < N; i++)
    if (is_root[i]) {
      lroots.push_back(int(i));
      for (auto& [col, c] : aff[i].coef) colpos.emplace(col, 0);
    }
  int J = 0;
  for (auto& [col, pos] : colpos) pos = J++;
  res.source_columns = J;
  res.rank = J;
  if (J == 0) return res;
  std::vector<int> src_of(J);
  for (auto& [col, pos] : colpos) src_of[pos] = col;
  std::vector<int> pivots, dependents;
  std::vector<std::vector<double>> M(J);  // M[d][m]: dependent column d on pivot m
  if (J >= 2 &&
      find_relations(d2, aff, lroots, colpos, dag.param_names().size(), param_defs, pivots, dependents, M)) {
    res.folded = true;
  } else {
    pivots.clear();
    dependents.clear();
    for (int j = 0; j < J; j++) pivots.push_back(j);
  }
  const int r = int(pivots.size());

  // Prepared columns and the rewritten DAG.
  res.cols.assign(r, {});
  for (int m = 0; m < r; m++) {
    res.cols[m].push_back({src_of[pivots[m]], 1.0});
    for (int d : dependents)
      if (M[d][m] != 0.0) res.cols[m].push_back({src_of[d], M[d][m]});
  }
  std::vector<int> in2(r);
  for (int m = 0; m < r; m++) in2[m] = d2.unary(Op::Input, m);
  // Without a fold the DAG keeps its structure; only input indices change.
  std::vector<int> pos_of(dag.input_names().size() + 1, -1);
  for (auto& [col, pos] : colpos) pos_of[col] = pos;
  std::vector<int> nw(N, -1);
  for (size_t i = 0; i < N; i++) {
    if (!live[i]) continue;
    if (kind[i] == K::Uniform) {
      nw[i] = copy_uniform(ns, int(i), d2, umemo);
      continue;
    }
    if (!res.folded && ns[i].op == Op::Input) {
      nw[i] = in2[pos_of[ns[i].index]];
      continue;
    }
    if (res.folded && kind[i] == K::Affine) {
      if (!is_root[i]) continue;
      int acc = -1;
      for (int m = 0; m < r; m++) {
        auto it = aff[i].coef.find(src_of[pivots[m]]);
        if (it == aff[i].coef.end()) continue;
        const Node& cn = d2.nodes()[it->second];
        if (cn.op == Op::Const && cn.value == 0.0) continue;
        const int term = d2.binary(Op::Mul, in2[m], it->second);
        acc = acc < 0 ? term : d2.binary(Op::Add, acc, term);
      }
      if (aff[i].cst >= 0) acc = acc < 0 ? aff[i].cst : d2.binary(Op::Add, acc, aff[i].cst);
      nw[i] = acc < 0 ? d2.constant(0.0) : acc;
      continue;
    }
    const Node& n = ns[i];
    auto m2 = [&](int c) { return c < 0 ? -1 : nw[c]; };
    switch (n.op) {
      case Op::Add: case Op::Sub: case Op::Mul: case Op::Div: case Op::Pow:
        nw[i] = d2.binary(n.op, m2(n.a), m2(n.b));
        break;
      case Op::Cmp: nw[i] = d2.compare(n.cmp, m2(n.a), m2(n.b)); break;
      case Op::Select: nw[i] = d2.select(m2(n.a), m2(n.b), m2(n.c)); break;
      default: nw[i] = d2.unary(n.op, m2(n.a)); break;
    }
    if (nw[i] < 0) throw std::runtime_error("fold: unmapped operand");
  }
  for (int rt : roots) res.roots.push_back(nw[rt]);
  res.rank = r;
  res.rewritten = true;
  res.dag = std::move(work);
  return res;
}

}  // namespace mf
