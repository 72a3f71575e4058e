// Lowering of MoreFit kernel expressions to CUDA C (see mf_lower.h).
#include "mf_lower.h"

#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <functional>
#include <set>
#include <sstream>
#include <stdexcept>

namespace mf {

namespace {

bool is_unary_fn(Op op) {
  switch (op) {
    case Op::Exp: case Op::Log: case Op::Sqrt: case Op::Sin: case Op::Cos: case Op::Tan:
    case Op::Asin: case Op::Acos: case Op::Atan: case Op::Erf:
      return true;
    default:
      return false;
  }
}

double apply_unary(Op op, double x) {
  switch (op) {
    case Op::Neg: return -x;
    case Op::Rcp: return 1.0 / x;
    case Op::Exp: return std::exp(x);
    case Op::Log: return std::log(x);
    case Op::Sqrt: return std::sqrt(x);
    case Op::Sin: return std::sin(x);
    case Op::Cos: return std::cos(x);
    case Op::Tan: return std::tan(x);
    case Op::Asin: return std::asin(x);
    case Op::Acos: return std::acos(x);
    case Op::Atan: return std::atan(x);
    case Op::Erf: return std::erf(x);
    default: throw std::runtime_error("not a unary op");
  }
}

double apply_binary(Op op, double a, double b) {
  switch (op) {
    case Op::Add: return a + b;
    case Op::Sub: return a - b;
    case Op::Mul: return a * b;
    case Op::Div: return a / b;
    case Op::Pow: return std::pow(a, b);
    default: throw std::runtime_error("not a binary op");
  }
}

bool apply_cmp(CmpOp c, double a, double b) {
  switch (c) {
    case CmpOp::Eq: return a == b;
    case CmpOp::Ne: return a != b;
    case CmpOp::Gt: return a > b;
    case CmpOp::Lt: return a < b;
    case CmpOp::Ge: return a >= b;
    case CmpOp::Le: return a <= b;
  }
  return false;
}

// ---------------------------------------------------------------- parser --
class Parser {
 public:
  Parser(Dag& dag, const std::string& s) : dag_(dag), s_(s) {}
  int run() {
    int r = expr();
    skip();
    if (p_ != s_.size()) fail("trailing characters");
    return r;
  }

 private:
  [[noreturn]] void fail(const std::string& what) {
    std::ostringstream m;
    m << "expression parse error (" << what << ") at offset " << p_ << " of \"" << s_.substr(0, 200)
      << (s_.size() > 200 ? "..." : "") << "\"";
    throw std::runtime_error(m.str());
  }
  void skip() {
    while (p_ < s_.size() && std::isspace((unsigned char)s_[p_])) p_++;
  }
  bool eat(const char* t) {
    skip();
    size_t n = std::strlen(t);
    if (s_.compare(p_, n, t) == 0) {
      p_ += n;
      return true;
    }
    return false;
  }
  int expr() {
    int c = comparison();
    if (eat("?")) {
      int a = expr();
      if (!eat(":")) fail("expected ':'");
      int b = expr();
      return dag_.select(c, a, b);
    }
    return c;
  }
  int comparison() {
    int a = additive();
    skip();
    static const struct { const char* t; CmpOp c; } ops[] = {{"==", CmpOp::Eq}, {"!=", CmpOp::Ne},
                                                             {">=", CmpOp::Ge}, {"<=", CmpOp::Le},
                                                             {">", CmpOp::Gt},  {"<", CmpOp::Lt}};
    for (auto& o : ops)
      if (eat(o.t)) return dag_.compare(o.c, a, additive());
    return a;
  }
  int additive() {
    int a = multiplicative();
    for (;;) {
      if (eat("+"))
        a = dag_.binary(Op::Add, a, multiplicative());
      else if (peek_binary_minus())
        a = dag_.binary(Op::Sub, a, multiplicative());
      else
        return a;
    }
  }
  bool peek_binary_minus() {
    skip();
    if (p_ < s_.size() && s_[p_] == '-') {
      p_++;
      return true;
    }
    return false;
  }
  int multiplicative() {
    int a = unary();
    for (;;) {
      if (eat("*"))
        a = dag_.binary(Op::Mul, a, unary());
      else if (eat("/"))
        a = dag_.binary(Op::Div, a, unary());
      else
        return a;
    }
  }
  int unary() {
    skip();
    if (eat("-")) return dag_.unary(Op::Neg, unary());
    if (eat("+")) return unary();
    return primary();
  }
  int primary() {
    skip();
    if (p_ >= s_.size()) fail("unexpected end");
    char ch = s_[p_];
    if (ch == '(') {
      p_++;
      int r = expr();
      if (!eat(")")) fail("expected ')'");
      return r;
    }
    if (std::isdigit((unsigned char)ch) || ch == '.') return number();
    if (std::isalpha((unsigned char)ch) || ch == '_') {
      size_t b = p_;
      while (p_ < s_.size() && (std::isalnum((unsigned char)s_[p_]) || s_[p_] == '_')) p_++;
      std::string id = s_.substr(b, p_ - b);
      skip();
      if (p_ < s_.size() && s_[p_] == '(') {
        p_++;
        std::vector<int> args;
        args.push_back(expr());
        while (eat(",")) args.push_back(expr());
        if (!eat(")")) fail("expected ')' after arguments");
        return call(id, args);
      }
      return variable(id);
    }
    fail(std::string("unexpected character '") + ch + "'");
  }
  int number() {
    const char* start = s_.c_str() + p_;
    char* end = nullptr;
    double v = std::strtod(start, &end);
    if (end == start) fail("bad number");
    p_ += size_t(end - start);
    return dag_.constant(v);
  }
  int call(const std::string& f, const std::vector<int>& a) {
    static const std::map<std::string, Op> fns = {
        {"exp", Op::Exp},   {"log", Op::Log},   {"sqrt", Op::Sqrt}, {"sin", Op::Sin},   {"cos", Op::Cos},
        {"tan", Op::Tan},   {"asin", Op::Asin}, {"acos", Op::Acos}, {"atan", Op::Atan}, {"erf", Op::Erf}};
    auto it = fns.find(f);
    if (it != fns.end()) {
      if (a.size() != 1) fail("wrong argument count for " + f);
      return dag_.unary(it->second, a[0]);
    }
    if (f == "pow") {
      if (a.size() != 2) fail("pow takes two arguments");
      return dag_.binary(Op::Pow, a[0], a[1]);
    }
    fail("unknown function " + f);
  }
  int variable(const std::string& id);

  Dag& dag_;
  const std::string& s_;
  size_t p_ = 0;
};

}  // namespace

// ------------------------------------------------------------------- DAG --
Dag::Dag(const std::vector<std::string>& inputs, const std::vector<std::string>& params)
    : inputs_(inputs), params_(params) {
  for (size_t i = 0; i < inputs.size(); i++) input_idx_[inputs[i]] = int(i);
  for (size_t i = 0; i < params.size(); i++)
    if (!param_idx_.count(params[i])) param_idx_[params[i]] = int(i);
}

int Parser::variable(const std::string& id) {
  // Input columns shadow parameters of the same name (the reference declares
  // parameters first and events inside the loop, compute_llvm.hh:601-646).
  auto& in = dag_.input_names();
  for (size_t i = 0; i < in.size(); i++)
    if (in[i] == id) return dag_.unary(Op::Input, int(i));
  auto& pa = dag_.param_names();
  for (size_t i = 0; i < pa.size(); i++)
    if (pa[i] == id) return dag_.unary(Op::Param, int(i));
  fail("unknown variable '" + id + "'");
}

int Dag::intern(const Node& n) {
  char key[160];
  uint64_t bits;
  std::memcpy(&bits, &n.value, sizeof bits);
  std::snprintf(key, sizeof key, "%d|%d|%llx|%d|%d|%d|%d", int(n.op), int(n.cmp), (unsigned long long)bits, n.index,
                n.a, n.b, n.c);
  auto it = table_.find(key);
  if (it != table_.end()) return it->second;
  nodes_.push_back(n);
  int id = int(nodes_.size()) - 1;
  table_[key] = id;
  return id;
}

int Dag::constant(double v) {
  Node n;
  n.op = Op::Const;
  n.value = v;
  return intern(n);
}

static bool is_const(const std::vector<Node>& ns, int id, double v) {
  return ns[id].op == Op::Const && ns[id].value == v;
}

int Dag::unary(Op op, int a) {
  if (op == Op::Input || op == Op::Param) {
    Node n;
    n.op = op;
    n.index = a;
    n.uniform = (op == Op::Param);
    return intern(n);
  }
  const Node& x = nodes_[a];
  if (x.op == Op::Const) return constant(apply_unary(op, x.value));
  if (op == Op::Neg && x.op == Op::Neg) return x.a;  // -(-y) = y exactly
  Node n;
  n.op = op;
  n.a = a;
  n.uniform = x.uniform;
  return intern(n);
}

int Dag::binary(Op op, int a, int b) {
  const Node& x = nodes_[a];
  const Node& y = nodes_[b];
  if (x.op == Op::Const && y.op == Op::Const) return constant(apply_binary(op, x.value, y.value));
  switch (op) {
    case Op::Add:
      if (y.op == Op::Neg) return binary(Op::Sub, a, y.a);  // a + (-b) = a - b exactly
      break;
    case Op::Mul:
      if (is_const(nodes_, b, 1.0)) return a;  // exact
      if (is_const(nodes_, a, 1.0)) return b;
      if (is_const(nodes_, b, -1.0)) return unary(Op::Neg, a);
      if (is_const(nodes_, a, -1.0)) return unary(Op::Neg, b);
      break;
    case Op::Div:
      if (is_const(nodes_, b, 1.0)) return a;
      // x / y -> x * (1/y): the reciprocal of a shared denominator (the
      // density in every gradient output) is computed once per event.
      if (is_const(nodes_, a, 1.0)) return unary(Op::Rcp, b);
      return binary(Op::Mul, a, unary(Op::Rcp, b));
    case Op::Pow:
      if (is_const(nodes_, b, 1.0)) return a;
      if (is_const(nodes_, b, 2.0)) return binary(Op::Mul, a, a);  // pow(x,2) and x*x round identically
      break;
    default:
      break;
  }
  Node n;
  n.op = op;
  n.a = a;
  n.b = b;
  n.uniform = x.uniform && y.uniform;
  return intern(n);
}

int Dag::compare(CmpOp c, int a, int b) {
  const Node& x = nodes_[a];
  const Node& y = nodes_[b];
  if (x.op == Op::Const && y.op == Op::Const) return constant(apply_cmp(c, x.value, y.value) ? 1.0 : 0.0);
  Node n;
  n.op = Op::Cmp;
  n.cmp = c;
  n.a = a;
  n.b = b;
  n.uniform = x.uniform && y.uniform;
  return intern(n);
}

int Dag::select(int cond, int a, int b) {
  const Node& c = nodes_[cond];
  if (c.op == Op::Const) return c.value != 0.0 ? a : b;
  if (a == b) return a;
  Node n;
  n.op = Op::Select;
  n.a = cond;
  n.b = a;
  n.c = b;
  n.uniform = c.uniform && nodes_[a].uniform && nodes_[b].uniform;
  return intern(n);
}

int Dag::parse(const std::string& expr) {
  Parser p(*this, expr);
  return p.run();
}

double Dag::eval(int id, const std::vector<double>& in, const std::vector<double>& pa) const {
  const Node& n = nodes_[id];
  switch (n.op) {
    case Op::Const: return n.value;
    case Op::Input: return in.at(n.index);
    case Op::Param: return pa.at(n.index);
    case Op::Add: case Op::Sub: case Op::Mul: case Op::Div: case Op::Pow:
      return apply_binary(n.op, eval(n.a, in, pa), eval(n.b, in, pa));
    case Op::Cmp: return apply_cmp(n.cmp, eval(n.a, in, pa), eval(n.b, in, pa)) ? 1.0 : 0.0;
    case Op::Select: return eval(n.a, in, pa) != 0.0 ? eval(n.b, in, pa) : eval(n.c, in, pa);
    default: return apply_unary(n.op, eval(n.a, in, pa));
  }
}

// -------------------------------------------------------------- emitter --
namespace {

std::string fmt_const(double v, bool f32) {
  char buf[64];
  if (std::isnan(v)) return f32 ? "__int_as_float(0x7fc00000)" : "__longlong_as_double(0x7ff8000000000000ULL)";
  if (std::isinf(v)) {
    if (f32) return v > 0 ? "__int_as_float(0x7f800000)" : "__int_as_float(0xff800000)";
    return v > 0 ? "__longlong_as_double(0x7ff0000000000000ULL)" : "__longlong_as_double(0xfff0000000000000ULL)";
  }
  if (f32)
    std::snprintf(buf, sizeof buf, "%.9ef", double(float(v)));
  else
    std::snprintf(buf, sizeof buf, "%.17e", v);
  std::string s(buf);
  return v < 0 ? "(" + s + ")" : s;
}

const char* fn_name(Op op, bool f32) {
  switch (op) {
    case Op::Exp: return f32 ? "expf" : "exp";
    case Op::Log: return f32 ? "logf" : "log";
    case Op::Sqrt: return f32 ? "sqrtf" : "sqrt";
    case Op::Sin: return f32 ? "sinf" : "sin";
    case Op::Cos: return f32 ? "cosf" : "cos";
    case Op::Tan: return f32 ? "tanf" : "tan";
    case Op::Asin: return f32 ? "asinf" : "asin";
    case Op::Acos: return f32 ? "acosf" : "acos";
    case Op::Atan: return f32 ? "atanf" : "atan";
    case Op::Erf: return f32 ? "erff" : "erf";
    case Op::Pow: return f32 ? "powf" : "pow";
    case Op::Rcp: return f32 ? "__frcp_rn" : "__drcp_rn";
    default: return "?";
  }
}

const char* cmp_str(CmpOp c) {
  switch (c) {
    case CmpOp::Eq: return "==";
    case CmpOp::Ne: return "!=";
    case CmpOp::Gt: return ">";
    case CmpOp::Lt: return "<";
    case CmpOp::Ge: return ">=";
    case CmpOp::Le: return "<=";
  }
  return "==";
}

// Marks the nodes reachable from `roots`.
std::vector<char> reachable(const std::vector<Node>& ns, const std::vector<int>& roots) {
  std::vector<char> r(ns.size(), 0);
  std::vector<int> st(roots.begin(), roots.end());
  while (!st.empty()) {
    int id = st.back();
    st.pop_back();
    if (id < 0 || r[id]) continue;
    r[id] = 1;
    const Node& n = ns[id];
    if (n.op == Op::Input || n.op == Op::Param || n.op == Op::Const) continue;
    st.push_back(n.a);
    st.push_back(n.b);
    st.push_back(n.c);
  }
  return r;
}

struct Emitter {
  const std::vector<Node>& ns;
  bool f32;  // arithmetic type float
  std::string T() const { return f32 ? "float" : "double"; }
  std::string ref(int id, const std::string& pfx) const {
    const Node& n = ns[id];
    if (n.op == Op::Const) return fmt_const(n.value, f32);
    if (n.op == Op::Input) return "x" + std::to_string(n.index);
    if (n.op == Op::Param) return "p" + std::to_string(n.index);
    return (n.uniform ? std::string("u") : pfx) + std::to_string(id);
  }
  // One SSA statement for node id (not for leaves).
  std::string stmt(int id, const std::string& pfx) const {
    const Node& n = ns[id];
    std::string lhs = "const " + std::string(n.op == Op::Cmp ? "bool" : T()) + " " + ref(id, pfx) + " = ";
    auto A = [&](int k) { return ref(k, pfx); };
    switch (n.op) {
      case Op::Add: return lhs + A(n.a) + " + " + A(n.b) + ";";
      case Op::Sub: return lhs + A(n.a) + " - " + A(n.b) + ";";
      case Op::Mul: return lhs + A(n.a) + " * " + A(n.b) + ";";
      case Op::Div: return lhs + A(n.a) + " / " + A(n.b) + ";";
      case Op::Neg: return lhs + "-" + A(n.a) + ";";
      case Op::Rcp: return lhs + fn_name(Op::Rcp, f32) + "(" + A(n.a) + ");";
      case Op::Pow: return lhs + fn_name(Op::Pow, f32) + "(" + A(n.a) + ", " + A(n.b) + ");";
      case Op::Cmp: return lhs + "(" + A(n.a) + " " + cmp_str(n.cmp) + " " + A(n.b) + ");";
      case Op::Select: return lhs + "(" + A(n.a) + " ? " + A(n.b) + " : " + A(n.c) + ");";
      default:
        if (is_unary_fn(n.op)) return lhs + fn_name(n.op, f32) + "(" + A(n.a) + ");";
        throw std::runtime_error("emit: unexpected node");
    }
  }
};

const char* kPrelude = R"CUDA(
typedef unsigned long long mf_u64;
#define MF_FULL 0xffffffffu
__device__ __forceinline__ double mf_warp_sum(double x) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(MF_FULL, x, o);
  return x;
}
// Neumaier-compensated add (fixed-order combine of block partials).
__device__ __forceinline__ void mf_neumaier(double& s, double& c, double x) {
  const double t = s + x;
  c += (fabs(s) >= fabs(x)) ? ((s - t) + x) : ((x - t) + s);
  s = t;
}
// Kahan step for FP32 per-thread partials (compute_llvm.hh:556-568 semantics).
__device__ __forceinline__ void mf_kahan_f32(float& s, float& c, float x) {
  const float y = __fsub_rn(x, c);
  const float t = __fadd_rn(s, y);
  c = __fsub_rn(__fsub_rn(t, s), y);
  s = t;
}
)CUDA";

}  // namespace

OpCount count_ops(const std::vector<std::string>& inputs, const std::vector<std::string>& params,
                  const std::vector<std::string>& exprs) {
  Dag dag(inputs, params);
  std::vector<int> roots;
  for (auto& e : exprs) roots.push_back(dag.parse(e));
  auto live = reachable(dag.nodes(), roots);
  OpCount c;
  for (size_t i = 0; i < dag.nodes().size(); i++) {
    if (!live[i]) continue;
    const Node& n = dag.nodes()[i];
    if (n.op == Op::Const || n.op == Op::Input || n.op == Op::Param) continue;
    c.nodes++;
    if (n.uniform) {
      c.uniform++;
      continue;
    }
    c.per_event++;
    if (is_unary_fn(n.op) || n.op == Op::Pow) c.transcendental++;
    if (n.op == Op::Rcp || n.op == Op::Div) c.divisions++;
  }
  return c;
}

LoweredKernel lower(const std::string& name, Kind kind, Elem elem, const std::vector<std::string>& inputs,
                    const std::vector<std::string>& params, const std::vector<std::string>& exprs,
                    const GenerateSpec* gen) {
  std::vector<std::string> in_names = inputs;
  if (kind == Kind::Generate) {
    if (!gen) throw std::runtime_error("generate kernel without generate spec");
    in_names = gen->dims;
  }
  Dag dag(in_names, params);
  std::vector<int> roots;
  for (auto& e : exprs) roots.push_back(dag.parse(e));
  const auto& ns = dag.nodes();
  auto live = reachable(ns, roots);

  const bool st32 = (elem == Elem::F32);
  // Arithmetic type: REDUCE kernels compute in the element type (the FP32
  // variant is the mixed-precision path); STORE kernels (event-only
  // precompute) compute in FP64 and round once on store; GENERATE kernels
  // compute in the element type like the reference's generate kernel.
  const bool ar32 = st32 && kind != Kind::Store;
  Emitter em{ns, ar32};
  const std::string ST = st32 ? "float" : "double";
  const std::string AT = ar32 ? "float" : "double";

  LoweredKernel out;
  out.entry = "mf_" + std::string(kind == Kind::Reduce ? "reduce" : kind == Kind::Store ? "store" : "generate");
  out.block = 256;
  out.vec = (kind == Kind::Generate) ? 1 : (st32 ? 4 : 2);
  const int V = out.vec;
  const int M = int(exprs.size());
  const int NP = std::max<int>(1, int(params.size()));

  std::set<int> used;
  for (size_t i = 0; i < ns.size(); i++)
    if (live[i] && ns[i].op == Op::Input) used.insert(ns[i].index);
  out.used_inputs.assign(used.begin(), used.end());

  std::ostringstream s;
  s << "// MoreFit CUDA backend: generated kernel '" << name << "' (" << (kind == Kind::Reduce ? "reduce"
                                                                          : kind == Kind::Store ? "store"
                                                                                                : "generate")
    << ", " << ST << " storage, " << AT << " arithmetic)\n";
  s << "// outputs:\n";
  for (size_t j = 0; j < exprs.size(); j++) s << "//   [" << j << "] " << exprs[j].substr(0, 160) << "\n";
  s << kPrelude;
  s << "#define MF_BLOCK " << out.block << "\n#define MF_NOUT " << M << "\n#define MF_NPAR " << NP << "\n";
  s << "struct mf_par { double v[MF_NPAR]; };\n";

  // Parameter-only prologue (u*), emitted once per thread.
  auto emit_params_and_uniform = [&](std::ostringstream& o, const std::string& src) {
    std::set<int> used_params;
    for (size_t i = 0; i < ns.size(); i++)
      if (live[i] && ns[i].op == Op::Param) used_params.insert(ns[i].index);
    for (int k : used_params) o << "  const " << AT << " p" << k << " = (" << AT << ")" << src << "[" << k << "];\n";
    for (size_t i = 0; i < ns.size(); i++) {
      if (!live[i] || !ns[i].uniform) continue;
      Op op = ns[i].op;
      if (op == Op::Const || op == Op::Param) continue;
      o << "  " << em.stmt(int(i), "u") << "\n";
    }
  };
  // Per-event body: x<k> already defined; defines e<id> and r<j>.
  auto emit_body = [&](std::ostringstream& o, const std::string& indent) {
    for (size_t i = 0; i < ns.size(); i++) {
      if (!live[i] || ns[i].uniform) continue;
      Op op = ns[i].op;
      if (op == Op::Input) continue;
      o << indent << em.stmt(int(i), "e") << "\n";
    }
    for (int j = 0; j < M; j++) o << indent << "const " << AT << " r" << j << " = " << em.ref(roots[j], "e") << ";\n";
  };

  if (kind == Kind::Reduce) {
    const std::string ACC = ar32 ? "float" : "double";
    // ---- single-dataset reduce ----
    s << "extern \"C\" __global__ void __launch_bounds__(MF_BLOCK) " << out.entry << "(const " << ST
      << "* __restrict__ data, mf_u64 stride, mf_u64 n, mf_par P, double* __restrict__ partials,"
      << " unsigned* __restrict__ counter, double* __restrict__ out) {\n";
    emit_params_and_uniform(s, "P.v");
    s << "  " << ACC << " acc[MF_NOUT];\n";
    if (ar32) s << "  float cmp[MF_NOUT];\n";
    s << "#pragma unroll\n  for (int j = 0; j < MF_NOUT; j++) { acc[j] = 0; " << (ar32 ? "cmp[j] = 0; " : "") << "}\n";
    s << "  const mf_u64 step = (mf_u64)gridDim.x * MF_BLOCK * " << V << ";\n";
    s << "  for (mf_u64 base = ((mf_u64)blockIdx.x * MF_BLOCK + threadIdx.x) * " << V
      << "; base < n; base += step) {\n";
    const std::string VT = st32 ? "float4" : "double2";
    for (int k : out.used_inputs)
      s << "    const " << VT << " l" << k << " = __ldg(reinterpret_cast<const " << VT << "*>(data + (mf_u64)" << k
        << " * stride + base));\n";
    const char* comp[4] = {"x", "y", "z", "w"};
    for (int v = 0; v < V; v++) {
      s << "    {\n";
      for (int k : out.used_inputs) s << "      const " << AT << " x" << k << " = l" << k << "." << comp[v] << ";\n";
      emit_body(s, "      ");
      s << "      if (base + " << v << " < n) {\n";
      for (int j = 0; j < M; j++) {
        if (ar32)
          s << "        mf_kahan_f32(acc[" << j << "], cmp[" << j << "], r" << j << ");\n";
        else
          s << "        acc[" << j << "] += r" << j << ";\n";
      }
      s << "      }\n    }\n";
    }
    s << "  }\n";
    // warp -> block -> grid, last block combines in fixed order
    s << R"CUDA(  __shared__ double red[MF_NOUT][MF_BLOCK / 32];
  __shared__ bool am_last;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int j = 0; j < MF_NOUT; j++) {
)CUDA";
    if (ar32)
      s << "    const double w = mf_warp_sum((double)acc[j] - (double)cmp[j]);\n";
    else
      s << "    const double w = mf_warp_sum(acc[j]);\n";
    s << R"CUDA(    if (lane == 0) red[j][warp] = w;
  }
  __syncthreads();
  for (int j = threadIdx.x; j < MF_NOUT; j += MF_BLOCK) {
    double b = 0.0;
#pragma unroll
    for (int w = 0; w < MF_BLOCK / 32; w++) b += red[j][w];
    partials[(mf_u64)blockIdx.x * MF_NOUT + j] = b;
  }
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) am_last = (atomicAdd(counter, 1u) == gridDim.x - 1);
  __syncthreads();
  if (!am_last) return;
  __threadfence();
  for (int j = warp; j < MF_NOUT; j += MF_BLOCK / 32) {
    double s = 0.0, c = 0.0;
    for (unsigned b = lane; b < gridDim.x; b += 32) mf_neumaier(s, c, __ldcg(partials + (mf_u64)b * MF_NOUT + j));
    double t = mf_warp_sum(s);
    double tc = mf_warp_sum(c);
    if (lane == 0) out[j] = t + tc;
  }
  if (threadIdx.x == 0) *counter = 0u;
}
)CUDA";

    // ---- ragged segments: one block per segment ----
    s << "extern \"C\" __global__ void __launch_bounds__(MF_BLOCK) " << out.entry << "_segments(const " << ST
      << "* __restrict__ data, mf_u64 stride, const mf_u64* __restrict__ seg_begin,"
      << " const unsigned* __restrict__ seg_count, const double* __restrict__ params, unsigned nparams,"
      << " double* __restrict__ out) {\n";
    s << "  const unsigned seg = blockIdx.x;\n  const mf_u64 first = seg_begin[seg];\n"
      << "  const mf_u64 cnt = seg_count[seg];\n  const double* __restrict__ Pv = params + (mf_u64)seg * nparams;\n";
    emit_params_and_uniform(s, "Pv");
    s << "  " << ACC << " acc[MF_NOUT];\n";
    if (ar32) s << "  float cmp[MF_NOUT];\n";
    s << "#pragma unroll\n  for (int j = 0; j < MF_NOUT; j++) { acc[j] = 0; " << (ar32 ? "cmp[j] = 0; " : "") << "}\n";
    s << "  for (mf_u64 i = threadIdx.x; i < cnt; i += MF_BLOCK) {\n";
    for (int k : out.used_inputs)
      s << "    const " << AT << " x" << k << " = (" << AT << ")__ldg(data + (mf_u64)" << k
        << " * stride + first + i);\n";
    emit_body(s, "    ");
    for (int j = 0; j < M; j++) {
      if (ar32)
        s << "    mf_kahan_f32(acc[" << j << "], cmp[" << j << "], r" << j << ");\n";
      else
        s << "    acc[" << j << "] += r" << j << ";\n";
    }
    s << "  }\n";
    s << R"CUDA(  __shared__ double red[MF_NOUT][MF_BLOCK / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int j = 0; j < MF_NOUT; j++) {
)CUDA";
    if (ar32)
      s << "    const double w = mf_warp_sum((double)acc[j] - (double)cmp[j]);\n";
    else
      s << "    const double w = mf_warp_sum(acc[j]);\n";
    s << R"CUDA(    if (lane == 0) red[j][warp] = w;
  }
  __syncthreads();
  for (int j = threadIdx.x; j < MF_NOUT; j += MF_BLOCK) {
    double b = 0.0, c = 0.0;
    for (int w = 0; w < MF_BLOCK / 32; w++) mf_neumaier(b, c, red[j][w]);
    out[(mf_u64)seg * MF_NOUT + j] = b + c;
  }
}
)CUDA";
  } else if (kind == Kind::Store) {
    s << "extern \"C\" __global__ void __launch_bounds__(MF_BLOCK) " << out.entry << "(const " << ST
      << "* __restrict__ data, mf_u64 stride, mf_u64 n, mf_par P, " << ST
      << "* __restrict__ outp, mf_u64 out_stride) {\n";
    emit_params_and_uniform(s, "P.v");
    s << "  const mf_u64 step = (mf_u64)gridDim.x * MF_BLOCK;\n";
    s << "  for (mf_u64 i = (mf_u64)blockIdx.x * MF_BLOCK + threadIdx.x; i < n; i += step) {\n";
    for (int k : out.used_inputs)
      s << "    const " << AT << " x" << k << " = (" << AT << ")data[(mf_u64)" << k << " * stride + i];\n";
    emit_body(s, "    ");
    for (int j = 0; j < M; j++) s << "    outp[(mf_u64)" << j << " * out_stride + i] = (" << ST << ")r" << j << ";\n";
    s << "  }\n}\n";
  } else {
    // GENERATE: one xoshiro128++ stream per thread, nper events per thread
    // (thread t owns events [t*nper, min((t+1)*nper, n))).
    const int D = int(gen->dims.size());
    s << R"CUDA(__device__ __forceinline__ unsigned mf_rotl(unsigned x, int k) { return (x << k) | (x >> (32 - k)); }
__device__ __forceinline__ unsigned mf_xoshiro(unsigned* s) {
  const unsigned r = mf_rotl(s[0] + s[3], 7) + s[0];
  const unsigned t = s[1] << 9;
  s[2] ^= s[0]; s[3] ^= s[1]; s[1] ^= s[2]; s[0] ^= s[3]; s[2] ^= t; s[3] = mf_rotl(s[3], 11);
  return r;
}
)CUDA";
    s << "extern \"C\" __global__ void __launch_bounds__(MF_BLOCK) " << out.entry
      << "(const unsigned* __restrict__ seeds, unsigned nseeds, mf_u64 n, mf_u64 nper, mf_par P, " << ST
      << "* __restrict__ outp, mf_u64 out_stride, unsigned* __restrict__ status, unsigned long long max_tries) {\n";
    s << "  const unsigned t = blockIdx.x * MF_BLOCK + threadIdx.x;\n  if (t >= nseeds) return;\n";
    s << "  unsigned st[4];\n#pragma unroll\n  for (int k = 0; k < 4; k++) st[k] = seeds[(mf_u64)k * nseeds + t];\n";
    emit_params_and_uniform(s, "P.v");
    // The reference prints min, max-min and maxprob with "%.15e" into its
    // generate kernel (compute_llvm.hh:466-478,485-489) and evaluates
    // min + delta*u and maxprob*u with one rounding per operation; the
    // explicit _rn intrinsics keep the compiler from fusing them, so the
    // proposals are bit-identical to the reference's.
    auto printed15 = [](double v) {
      char b[64];
      std::snprintf(b, sizeof b, "%.15e", v);
      return std::strtod(b, nullptr);
    };
    const char* mul = ar32 ? "__fmul_rn" : "__dmul_rn";
    const char* add = ar32 ? "__fadd_rn" : "__dadd_rn";
    s << "  const " << AT << " maxprob = " << fmt_const(printed15(gen->maxprob), ar32) << ";\n";
    s << "  const mf_u64 from = (mf_u64)t * nper;\n  mf_u64 to = from + nper; if (to > n) to = n;\n";
    s << "  unsigned long long tries = 0;\n";
    s << "  for (mf_u64 i = from; i < to; i++) {\n    for (;;) {\n";
    s << "      if (++tries > max_tries) { atomicOr(status, 1u); return; }\n";
    for (int d = 0; d < D; d++) {
      s << "      const " << AT << " x" << d << " = " << add << "(" << fmt_const(printed15(gen->lo[d]), ar32) << ", "
        << mul << "(" << fmt_const(printed15(gen->hi[d] - gen->lo[d]), ar32) << ", (" << AT
        << ")(mf_xoshiro(st) * 2.3283064365386963e-10)));\n";
    }
    emit_body(s, "      ");
    s << "      if (" << mul << "(maxprob, (" << AT << ")(mf_xoshiro(st) * 2.3283064365386963e-10)) < r0) {\n";
    for (int d = 0; d < D; d++) s << "        outp[(mf_u64)" << d << " * out_stride + i] = (" << ST << ")x" << d << ";\n";
    s << "        break;\n      }\n    }\n  }\n}\n";
  }
  out.source = s.str();
  return out;
}

}  // namespace mf
