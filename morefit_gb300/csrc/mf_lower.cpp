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

// REDUCE kernels with more than kAccRegMax outputs keep the per-thread
// partials of as many outputs as fit in kAccSmemBytes of shared memory per
// block there (the last ones), and at least kAccRegMin in registers.
constexpr int kAccRegMax = 64, kAccRegMin = 8;
constexpr size_t kAccSmemBytes = 40 * 1024;

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

void Dag::eval_all(const double* pa, size_t np, std::vector<double>& v) const {
  v.resize(nodes_.size());
  for (size_t i = 0; i < nodes_.size(); i++) {
    const Node& n = nodes_[i];
    switch (n.op) {
      case Op::Const: v[i] = n.value; break;
      case Op::Input: v[i] = 0.0; break;
      case Op::Param: v[i] = size_t(n.index) < np ? pa[n.index] : 0.0; break;
      case Op::Add: case Op::Sub: case Op::Mul: case Op::Div: case Op::Pow:
        v[i] = apply_binary(n.op, v[n.a], v[n.b]);
        break;
      case Op::Cmp: v[i] = apply_cmp(n.cmp, v[n.a], v[n.b]) ? 1.0 : 0.0; break;
      case Op::Select: v[i] = v[n.a] != 0.0 ? v[n.b] : v[n.c]; break;
      default: v[i] = apply_unary(n.op, v[n.a]); break;
    }
  }
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
      case Op::Exp:
      case Op::Log:
      case Op::Sqrt:
      case Op::Sin:
      case Op::Cos: return lhs + fn_name(n.op, f32) + "(" + A(n.a) + ");";
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
// Programmatic dependent launch (PTX griddepcontrol): no-ops unless the grid
// was launched with programmatic stream serialization.
__device__ __forceinline__ void mf_launch_dependents() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }
__device__ __forceinline__ void mf_grid_dependency_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
// Device-scope fetch-and-add with acquire-release semantics.
__device__ __forceinline__ unsigned mf_atom_add_acq_rel(unsigned* p, unsigned v) {
  unsigned old;
  asm volatile("atom.acq_rel.gpu.global.add.u32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(v) : "memory");
  return old;
}
// Kahan step for FP32 per-thread partials (compute_llvm.hh:556-568 semantics).
__device__ __forceinline__ void mf_kahan_f32(float& s, float& c, float x) {
  const float y = __fsub_rn(x, c);
  const float t = __fadd_rn(s, y);
  c = __fsub_rn(__fsub_rn(t, s), y);
  s = t;
}
)CUDA";

// Double-float ("double-word") arithmetic on pairs of FP32 values, used by
// FP64 REDUCE kernels. GB300 issues FP32 at 64x its FP64 rate; a value is
// kept as an unevaluated sum h + l of two floats (|l| <= ulp(h)/2, ~48
// significant bits) and combined with error-free transforms: TwoSum (Knuth),
// FastTwoSum (Dekker 1971) and the FMA-based TwoProd; addition and
// multiplication follow the double-word algorithms analysed by Joldes, Muller
// and Popescu (ACM TOMS 44, 2017). The logarithm is table driven in the manner
// of Tang (ACM TOMS 16, 1990): log y = E ln2 + ln c_j + ln(1+t) with c_j the
// centre of one of 128 mantissa intervals, |t| <= 2^-8 and a short series.
// Operations without a double-float form fall back to FP64 on the value.
const char* kDwPrelude = R"CUDA(
struct mf_dw { float h, l; };
__device__ __forceinline__ mf_dw mf_dw_make(float h, float l) { mf_dw r; r.h = h; r.l = l; return r; }
__device__ __forceinline__ mf_dw mf_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  return mf_dw_make(s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb)));
}
__device__ __forceinline__ mf_dw mf_fast_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  return mf_dw_make(s, __fsub_rn(b, __fsub_rn(s, a)));
}
__device__ __forceinline__ mf_dw mf_dw_add(mf_dw a, mf_dw b) {
  const mf_dw s = mf_two_sum(a.h, b.h);
  return mf_fast_two_sum(s.h, __fadd_rn(__fadd_rn(a.l, b.l), s.l));
}
__device__ __forceinline__ mf_dw mf_dw_neg(mf_dw a) { return mf_dw_make(-a.h, -a.l); }
__device__ __forceinline__ mf_dw mf_dw_sub(mf_dw a, mf_dw b) { return mf_dw_add(a, mf_dw_neg(b)); }
__device__ __forceinline__ mf_dw mf_dw_mul(mf_dw a, mf_dw b) {
  const float p = __fmul_rn(a.h, b.h);
  const float e = __fmaf_rn(a.h, b.l, __fmaf_rn(a.l, b.h, __fmaf_rn(a.h, b.h, -p)));
  return mf_fast_two_sum(p, e);
}
__device__ __forceinline__ mf_dw mf_dw_rcp(mf_dw a) {
  // r = 1/a.h, then one Newton correction with the residual 1 - a*r formed exactly to first order.
  const float r = __frcp_rn(a.h);
  const float p = __fmul_rn(a.h, r);
  const float pe = __fmaf_rn(a.h, r, -p);
  const float e = __fsub_rn(__fsub_rn(__fsub_rn(1.0f, p), pe), __fmul_rn(a.l, r));
  return mf_fast_two_sum(r, __fmul_rn(r, e));
}
// An infinite high word is the value (its low word is NaN after inf - inf
// in the error terms of a sum).
__device__ __forceinline__ double mf_dw_to_double(mf_dw a) {
  return isinf(a.h) ? (double)a.h : (double)a.h + (double)a.l;
}
__device__ __forceinline__ mf_dw mf_dw_from_double(double x) {
  const float h = __double2float_rn(x);
  return mf_dw_make(h, __double2float_rn(x - (double)h));
}
// Splits an FP64 value into h + l with integer and FP32 operations only (no
// FP64 pipe, no conversion instructions, no branch): h keeps the top 24
// significand bits (truncated), l the next 23. Magnitudes below 2^-126 give
// h = l = 0 (an absolute error below 1.2e-38), l underflows to 0 below
// 2^-81, magnitudes from 2^128 on give +-inf, NaN stays NaN.
__device__ __forceinline__ mf_dw mf_dw_split(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const unsigned hi32 = (unsigned)(b >> 32), lo32 = (unsigned)b;
  const unsigned e = (hi32 >> 20) & 0x7ffu;
  const unsigned sign = hi32 & 0x80000000u;
  const unsigned hnorm = sign | ((e - 896u) << 23) | ((hi32 & 0xfffffu) << 3) | (lo32 >> 29);
  const unsigned hbig = sign | 0x7f800000u | ((e == 2047u && ((hi32 & 0xfffffu) | lo32)) ? 0x400000u : 0u);
  const unsigned hb = e > 1150u ? hbig : (e >= 897u ? hnorm : sign);
  // top 23 of the 29 remaining bits as an exact float (exponent-field trick), scaled by 2^(e - 1069)
  const float r23 = __fsub_rn(__uint_as_float(0x4b000000u | ((lo32 & 0x1fffffffu) >> 6)), 8388608.0f);
  const unsigned sb = (e >= 943u && e <= 1150u) ? ((e - 942u) << 23) : 0u;
  const float l = __fmul_rn(r23, __uint_as_float(sb));
  return mf_dw_make(__uint_as_float(hb), __uint_as_float(__float_as_uint(l) | sign));
}
__device__ __forceinline__ mf_dw mf_dw_pair(float2 t) { return mf_dw_make(t.x, t.y); }
// Lazy double-float accumulation (per-thread partials, dot products): TwoSum
// of the high words, the low words and the rounding error added in FP32;
// mf_dw_renorm restores a normalized pair (|l| <= ulp(h)/2) at the end.
__device__ __forceinline__ void mf_dw_acc(mf_dw& a, mf_dw x) {
  const mf_dw s = mf_two_sum(a.h, x.h);
  a.h = s.h;
  a.l = __fadd_rn(a.l, __fadd_rn(s.l, x.l));
}
// a += x * y (the product's error terms formed with FMA, as in mf_dw_mul)
__device__ __forceinline__ void mf_dw_acc_mul(mf_dw& a, mf_dw x, mf_dw y) {
  const float p = __fmul_rn(x.h, y.h);
  const float e = __fmaf_rn(x.h, y.l, __fmaf_rn(x.l, y.h, __fmaf_rn(x.h, y.h, -p)));
  const mf_dw s = mf_two_sum(a.h, p);
  a.h = s.h;
  a.l = __fadd_rn(a.l, __fadd_rn(s.l, e));
}
// a += x * y for FP32 operands: the product is exact as p + e (FMA), so a
// dot product of FP32 values accumulated this way is as accurate as one
// computed in double-float (the compensated dot product of Ogita, Rump and
// Oishi, SIAM J. Sci. Comput. 26, 2005, with a lazily renormalised sum).
__device__ __forceinline__ mf_dw mf_dw_prodf(float x, float y) {
  const float p = __fmul_rn(x, y);
  return mf_dw_make(p, __fmaf_rn(x, y, -p));
}
// The same with a double-float factor c = c.h + c.l (a parameter-only
// coefficient kept to ~48 bits): x * c.h exact as p + e, plus x * c.l.
__device__ __forceinline__ mf_dw mf_dw_prodfw(float x, mf_dw c) {
  const float p = __fmul_rn(x, c.h);
  return mf_dw_make(p, __fmaf_rn(x, c.l, __fmaf_rn(x, c.h, -p)));
}
__device__ __forceinline__ void mf_dw_acc_mulfw(mf_dw& a, float x, mf_dw c) {
  const float p = __fmul_rn(x, c.h);
  const float e = __fmaf_rn(x, c.l, __fmaf_rn(x, c.h, -p));
  const mf_dw s = mf_two_sum(a.h, p);
  a.h = s.h;
  a.l = __fadd_rn(a.l, __fadd_rn(s.l, e));
}
__device__ __forceinline__ void mf_dw_acc_mulf(mf_dw& a, float x, float y) {
  const float p = __fmul_rn(x, y);
  const float e = __fmaf_rn(x, y, -p);
  const mf_dw s = mf_two_sum(a.h, p);
  a.h = s.h;
  a.l = __fadd_rn(a.l, __fadd_rn(s.l, e));
}
__device__ __forceinline__ mf_dw mf_dw_renorm(mf_dw a) { return mf_two_sum(a.h, a.l); }
// Round-to-nearest split with integer operations only: h = x rounded to 24
// bits, l = x - h rounded to 24 bits, |x - h - l| <= 2^-48 |x| for |x| from
// 2^-100 to 2^127 (below 2^-100 l loses bits to the FP32 exponent range).
// Magnitudes outside [2^-126, 2^127) (and zero, inf, NaN) take the
// truncating split. No FP64 instruction on any path: a short FP64 fallback
// would be if-converted and executed for every value.
__device__ __forceinline__ mf_dw mf_dw_split_rn(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const unsigned e = (unsigned)(b >> 52) & 0x7ffu;
  if (e < 897u || e > 1149u) return mf_dw_split(x);
  const unsigned sign = (unsigned)(b >> 32) & 0x80000000u;
  const unsigned long long M = (b & 0xfffffffffffffull) | 0x10000000000000ull;  // 53-bit significand
  const unsigned long long H = (M + 0x10000000ull) >> 29;                       // nearest 24-bit value
  const long long L = (long long)M - (long long)(H << 29);                      // |L| <= 2^28
  const unsigned carry = (unsigned)(H >> 24);                                   // H = 2^24: next binade
  const float h = __uint_as_float(sign | ((e - 896u + carry) << 23) | (carry ? 0u : ((unsigned)H & 0x7fffffu)));
  const unsigned al = (unsigned)(L < 0 ? -L : L);
  // |L| rounded to its top 24 bits as an exact float (exponent-field trick),
  // scaled by 2^(e - 1070) (as 2^(e - 1006) * 2^-64 where e - 1070 < -126)
  const float m = __fsub_rn(__uint_as_float(0x4b000000u | ((al + 16u) >> 5)), 8388608.0f);
  const bool low = e < 944u;
  const float lm = __fmul_rn(__fmul_rn(m, __uint_as_float((low ? e - 879u : e - 943u) << 23)),
                             low ? 0x1p-64f : 1.0f);
  return mf_dw_make(h, __uint_as_float(__float_as_uint(lm) | (sign ^ (L < 0 ? 0x80000000u : 0u))));
}
// h + l as an FP64 value with integer operations only: h's significand
// extended by l's bits down to the double's last place (l's bits below it
// are dropped, an error below one unit in the last place). The pair is
// renormalized first; zero or subnormal h gives a signed zero (an absolute
// error below 2^-125), inf and NaN carry over.
__device__ __forceinline__ double mf_dw_to_double_bits(mf_dw a) {
  a = mf_fast_two_sum(a.h, a.l);
  const unsigned hb = __float_as_uint(a.h), lb = __float_as_uint(a.l);
  const int eh = (int)((hb >> 23) & 0xffu), el = (int)((lb >> 23) & 0xffu);
  const int k = 29 + el - eh;  // scale of l's significand in units of the double's last place (<= 5)
  if (eh == 0 || eh == 255)
    return __longlong_as_double((long long)(((unsigned long long)(hb >> 31) << 63) |
                                            (eh ? (0x7ffull << 52) | ((hb & 0x7fffffu) ? (1ull << 51) : 0ull) : 0ull)));
  unsigned long long M = (unsigned long long)((hb & 0x7fffffu) | 0x800000u) << 29;
  int E = eh;
  if (el != 0) {
    const unsigned long long ml = (lb & 0x7fffffu) | 0x800000u;
    const unsigned long long v = k >= 0 ? (ml << k) : (k > -40 ? (ml >> -k) : 0ull);
    if ((hb ^ lb) >> 31) {
      M -= v;
      if (M < (1ull << 52)) { M <<= 1; E -= 1; }
    } else {
      M += v;
      if (M >= (1ull << 53)) { M >>= 1; E += 1; }
    }
  }
  return __longlong_as_double((long long)(((unsigned long long)(hb >> 31) << 63) |
                                          ((unsigned long long)(E + 896) << 52) | (M & 0xfffffffffffffull)));
}
__device__ __forceinline__ mf_dw mf_dw_mulf(mf_dw a, float b) {
  const float p = __fmul_rn(a.h, b);
  return mf_fast_two_sum(p, __fmaf_rn(a.l, b, __fmaf_rn(a.h, b, -p)));
}
// Square root: the correctly rounded FP32 root s of a.h, corrected by the
// series sqrt(s^2 + r) = s + d - d^2/(2s) + ..., d = r/(2s). d reaches
// 2^-23 s, so the residual r = a - s^2 (s^2 exact by FMA) and d are kept as
// double-float values; the next term, d^3/(2s^2), is below 2^-70 s.
// sqrt(0) = 0, negative or NaN -> NaN, +inf -> +inf.
__device__ __forceinline__ mf_dw mf_dw_sqrt(mf_dw a) {
  if (!(a.h > 0.0f) || a.h == __int_as_float(0x7f800000))
    return mf_dw_make(a.h == 0.0f ? 0.0f : (a.h > 0.0f ? a.h : __int_as_float(0x7fc00000)), 0.0f);
  const float s = __fsqrt_rn(a.h);
  const float p = __fmul_rn(s, s);
  const float pe = __fmaf_rn(s, s, -p);
  // a.h - p is exact (Sterbenz); the rest of the residual in double-float
  const mf_dw r = mf_dw_add(mf_two_sum(__fsub_rn(a.h, p), -pe), mf_dw_make(a.l, 0.0f));
  const float s2 = __fadd_rn(s, s);
  const float dh = __fdiv_rn(r.h, s2);
  const float dl = __fdiv_rn(__fadd_rn(__fmaf_rn(-dh, s2, r.h), r.l), s2);
  const float q = __fdiv_rn(__fmul_rn(dh, dh), s2);
  const mf_dw t = mf_fast_two_sum(s, dh);
  return mf_fast_two_sum(t.h, __fadd_rn(t.l, __fsub_rn(dl, q)));
}
// sin and cos of a double-float. a = k*(pi/2) + r, |r| <~ pi/4, by a
// four-part Cody-Waite reduction: pi/2 = C1 + C2 + C3 + C4 with C1 and C2 of
// 12 significant bits (k*C1, k*C2 exact for |k| < 2^12) and a remainder below
// 4e-22. sin r and cos r are their Taylor series, the terms above 2^-26 in
// double-float (Horner), the rest in FP32; the first omitted term is below
// 2e-16 relative. Arguments beyond |a| = 6000 (and inf/NaN) use FP64.
__device__ __forceinline__ void mf_dw_sincos(mf_dw a, mf_dw* sn, mf_dw* cs) {
  if (!(fabsf(a.h) <= 6000.0f)) {
    const double x = mf_dw_to_double(a);
    *sn = mf_dw_from_double(sin(x));
    *cs = mf_dw_from_double(cos(x));
    return;
  }
  const float k = rintf(__fmul_rn(a.h, 0x1.45f306p-1f));
  const float t1 = __fmaf_rn(-k, 0x1.92p+0f, a.h);  // exact
  mf_dw r = mf_two_sum(t1, -__fmul_rn(k, 0x1.fb4p-12f));
  const float p3 = __fmul_rn(k, 0x1.4442dp-24f);
  r = mf_dw_sub(r, mf_dw_make(p3, __fmaf_rn(k, 0x1.4442dp-24f, -p3)));
  r = mf_dw_add(r, mf_dw_make(__fmaf_rn(-k, 0x1.846988p-48f, a.l), 0.0f));
  const mf_dw r2 = mf_dw_mul(r, r);
  const float z = r2.h;
  // sin r = r + r^3 (c3 + r^2 (c5 + r^2 (c7 + r^2 (c9 + r^2 T)))), c_n = (-1)^((n-1)/2) / n!
  const float T = __fmaf_rn(z, __fmaf_rn(z, -0x1.ae7f3ep-41f, 0x1.612462p-33f), -0x1.ae6456p-26f);
  mf_dw q = mf_dw_add(mf_dw_make(0x1.71de3ap-19f, 0x1.55b1ccp-45f), mf_dw_mulf(r2, T));
  q = mf_dw_add(mf_dw_make(-0x1.a01a02p-13f, 0x1.7f97fap-39f), mf_dw_mul(r2, q));
  q = mf_dw_add(mf_dw_make(0x1.111112p-7f, -0x1.dddddep-32f), mf_dw_mul(r2, q));
  q = mf_dw_add(mf_dw_make(-0x1.555556p-3f, 0x1.555556p-28f), mf_dw_mul(r2, q));
  const mf_dw sr = mf_dw_add(r, mf_dw_mul(mf_dw_mul(r, r2), q));
  // cos r = 1 + r^2 (c2 + r^2 (c4 + r^2 (c6 + r^2 (c8 + r^2 (c10 + r^2 T2))))), c_n = (-1)^(n/2) / n!
  const float T2 = __fmaf_rn(z, __fmaf_rn(z, 0x1.ae7f3ep-45f, -0x1.93974ap-37f), 0x1.1eed8ep-29f);
  mf_dw u = mf_dw_add(mf_dw_make(-0x1.27e4fcp-22f, 0x1.10ec14p-47f), mf_dw_mulf(r2, T2));
  u = mf_dw_add(mf_dw_make(0x1.a01a02p-16f, -0x1.7f97fap-42f), mf_dw_mul(r2, u));
  u = mf_dw_add(mf_dw_make(-0x1.6c16c2p-10f, 0x1.27d27ep-35f), mf_dw_mul(r2, u));
  u = mf_dw_add(mf_dw_make(0x1.555556p-5f, -0x1.555556p-30f), mf_dw_mul(r2, u));
  u = mf_dw_add(mf_dw_make(-0.5f, 0.0f), mf_dw_mul(r2, u));
  const mf_dw cr = mf_dw_add(mf_dw_make(1.0f, 0.0f), mf_dw_mul(r2, u));
  const int quad = ((int)k) & 3;
  const mf_dw s0 = (quad & 1) ? cr : sr, c0 = (quad & 1) ? sr : cr;
  *sn = (quad & 2) ? mf_dw_neg(s0) : s0;
  *cs = ((quad + 1) & 2) ? mf_dw_neg(c0) : c0;
}
__device__ __forceinline__ mf_dw mf_dw_sin(mf_dw a) { mf_dw s, c; mf_dw_sincos(a, &s, &c); return s; }
__device__ __forceinline__ mf_dw mf_dw_cos(mf_dw a) { mf_dw s, c; mf_dw_sincos(a, &s, &c); return c; }
// ln of a positive double-float (see above); zero gives -inf, negative or
// NaN gives NaN, +inf gives +inf, subnormal h is rescaled by 2^64 first.
__device__ __forceinline__ mf_dw mf_dw_log(mf_dw a, const float4* __restrict__ tab) {
  const bool sub = a.h > 0.0f && a.h < 1.17549435e-38f;
  const float ah = sub ? __fmul_rn(a.h, 18446744073709551616.0f) : a.h;
  const float al = sub ? __fmul_rn(a.l, 18446744073709551616.0f) : a.l;
  const unsigned bits = __float_as_uint(ah);
  const int E = (int)((bits >> 23) & 0xffu) - 127;
  const float m = __uint_as_float((bits & 0x007fffffu) | 0x3f800000u);
  const float4 T = tab[(bits >> 16) & 0x7fu];  // {ln c hi, ln c lo, 1/c, c}
  const unsigned se = (unsigned)(127 - E);
  const float yl = __fmul_rn(al, __uint_as_float(se >= 1u && se <= 254u ? (se << 23) : 0u));
  const mf_dw N = mf_two_sum(__fsub_rn(m, T.w), yl);
  const float th = __fmul_rn(N.h, T.z);
  const float tl = __fmul_rn(__fadd_rn(__fmaf_rn(-th, T.w, N.h), N.l), T.z);
  const float sh = __fmul_rn(th, th);
  const float sl = __fmaf_rn(2.0f * th, tl, __fmaf_rn(th, th, -sh));
  mf_dw lt = mf_dw_sub(mf_dw_make(th, tl), mf_dw_make(0.5f * sh, 0.5f * sl));
  const float P = __fmaf_rn(th, __fmaf_rn(th, __fmaf_rn(th, __fmaf_rn(th, 0.142857143f, -0.166666667f), 0.2f), -0.25f),
                            0.333333333f);
  lt = mf_dw_add(lt, mf_dw_make(__fmul_rn(__fmul_rn(sh, th), P), 0.0f));
  const int Et = E - (sub ? 64 : 0);
  const float Ef = __fsub_rn(__int_as_float(0x4b400000 + Et), 12582912.0f);  // (float)Et without a conversion
  // E*ln2 with ln2 = L1 + L2 + L3 (L1 of 12 bits: E*L1 exact; remainder of L3 below 1e-19)
  const float e1 = __fmul_rn(Ef, 0x1.62ep-1f);
  const float e2 = __fmul_rn(Ef, 0x1.0bfbe8p-15f);
  const mf_dw e12 = mf_two_sum(e1, e2);
  const mf_dw el = mf_fast_two_sum(
      e12.h, __fadd_rn(e12.l, __fmaf_rn(Ef, 0x1.cf79aap-40f, __fmaf_rn(Ef, 0x1.0bfbe8p-15f, -e2))));
  mf_dw r = mf_dw_add(mf_dw_add(el, mf_dw_make(T.x, T.y)), lt);
  const float inf = __uint_as_float(0x7f800000u);
  if (a.h == 0.0f) r = mf_dw_make(-inf, 0.0f);
  if (!(a.h >= 0.0f)) r = mf_dw_make(__uint_as_float(0x7fc00000u), 0.0f);
  if (a.h == inf) r = mf_dw_make(inf, 0.0f);
  return r;
}
// exp of a double-float value by Tang's table-driven method (P. T. P. Tang,
// ACM TOMS 15 (1989) 144-157): x = (64k + j) ln2/64 + r with ln2/64 split as
// C1 + C2 + C3 (C1 of 9 significant bits, so N*C1 is exact for |N| < 2^13),
// |r| <= ln2/128 (+ a rounding); exp(r) - 1 = r + r^2/2 + r^3/6 in
// double-float plus r^4/24 + r^5/120 + r^6/720 in FP32 (below 4e-11);
// exp(x) = 2^k * T_j * (1 + (exp(r) - 1)) with T_j = 2^(j/64) from the table,
// 2^k applied as two exact power-of-two factors. Relative error ~2^-46 for
// results from 2^-100 to 2^128 (where the low word is a normal float); below
// 2^-100 the low word loses bits (an absolute error of a few 2^-149, the
// resolution of any double-float value there) and results under 2^-149 are
// 0; above 2^128 the result is +inf; NaN stays NaN.
__device__ __forceinline__ mf_dw mf_dw_exp(mf_dw a, const float2* __restrict__ tab) {
  const float x = fminf(fmaxf(a.h, -104.0f), 89.0f);
  // N = x * 64/ln2 rounded to an integer (|N| < 2^14) without a conversion:
  // adding 1.5*2^23 leaves the integer in the low significand bits
  const float tn = __fmaf_rn(x, 0x1.715476p+6f, 12582912.0f);
  const int Ni = __float_as_int(tn) - 0x4b400000;
  const float N = __fsub_rn(tn, 12582912.0f);
  const int j = Ni & 63;
  const int k = (Ni - j) >> 6;
  const float t1 = __fmaf_rn(-N, 0x1.63p-7f, x);  // exact
  const float p2 = __fmul_rn(N, -0x1.bd0106p-19f);
  const float p2e = __fmaf_rn(N, -0x1.bd0106p-19f, -p2);
  mf_dw r = mf_two_sum(t1, -p2);
  r = mf_fast_two_sum(r.h, __fadd_rn(r.l, __fsub_rn(__fmaf_rn(-N, 0x1.cf79acp-46f, a.l), p2e)));
  const mf_dw r2 = mf_dw_mul(r, r);
  const mf_dw r3 = mf_dw_mul(r2, r);
  mf_dw t3 = mf_dw_mul(r3, mf_dw_make(0x1.555556p-3f, -0x1.555556p-28f));
  const float q = __fmul_rn(__fmul_rn(r2.h, r2.h),
                            __fmaf_rn(r.h, __fmaf_rn(r.h, 0x1.6c16c2p-10f, 0x1.111112p-7f), 0x1.555556p-5f));
  t3 = mf_fast_two_sum(t3.h, __fadd_rn(t3.l, q));
  mf_dw e = mf_dw_add(r, mf_dw_make(0.5f * r2.h, 0.5f * r2.l));
  e = mf_dw_add(e, t3);
  const float2 T = tab[j];
  const mf_dw Tj = mf_dw_make(T.x, T.y);
  mf_dw y = mf_dw_add(Tj, mf_dw_mul(Tj, e));
  const int k1 = k >> 1, k2 = k - k1;  // both in [-76, 64]
  const float s1 = __int_as_float((k1 + 127) << 23), s2 = __int_as_float((k2 + 127) << 23);
  y = mf_dw_make(__fmul_rn(__fmul_rn(y.h, s1), s2), __fmul_rn(__fmul_rn(y.l, s1), s2));
  if (a.h > 89.0f) y = mf_dw_make(__int_as_float(0x7f800000), 0.0f);
  if (a.h < -104.0f) y = mf_dw_make(0.0f, 0.0f);
  if (a.h != a.h) y = mf_dw_make(a.h, a.h);
  return y;
}
// a^b = exp(b ln|a|) in double-float. a < 0: for integer b the sign follows
// b's parity, otherwise NaN; a = 0: 0 for b > 0, +inf for b < 0; b = 0: 1
// (also for a NaN). Relative error ~|b ln a| 2^-46.
__device__ __forceinline__ mf_dw mf_dw_pow(mf_dw a, mf_dw b, const float4* __restrict__ ltab,
                                           const float2* __restrict__ etab) {
  const bool neg = a.h < 0.0f;
  const mf_dw aa = neg ? mf_dw_neg(a) : a;
  mf_dw r = mf_dw_exp(mf_dw_mul(b, mf_dw_log(aa, ltab)), etab);
  // integer b and its parity from the significand bits (|v| < 2^23: v + 2^23
  // holds v's integer part in its last bits; |v| >= 2^23 is an integer)
  const float bh = fabsf(b.h), bl = fabsf(b.l);
  const float th = __fadd_rn(bh, 8388608.0f), tl = __fadd_rn(bl, 8388608.0f);
  const bool int_h = bh >= 8388608.0f || __fsub_rn(th, 8388608.0f) == bh;
  const bool int_l = bl >= 8388608.0f || __fsub_rn(tl, 8388608.0f) == bl;
  const bool int_b = int_h && int_l;
  const bool odd = bh < 8388608.0f ? (__float_as_int(th) & 1) != 0
                                   : (bh < 16777216.0f ? (__float_as_int(b.h) & 1) != 0
                                                       : (bl < 8388608.0f && (__float_as_int(tl) & 1) != 0));
  if (neg) r = int_b ? (odd ? mf_dw_neg(r) : r) : mf_dw_make(__int_as_float(0x7fc00000), 0.0f);
  if (a.h == 0.0f) r = mf_dw_make(b.h > 0.0f ? 0.0f : __int_as_float(0x7f800000), 0.0f);
  if (b.h == 0.0f) r = mf_dw_make(1.0f, 0.0f);
  return r;
}
// Comparisons of normalized double-float values (lexicographic on (h, l)).
__device__ __forceinline__ bool mf_dw_gt(mf_dw a, mf_dw b) { return a.h > b.h || (a.h == b.h && a.l > b.l); }
__device__ __forceinline__ bool mf_dw_lt(mf_dw a, mf_dw b) { return a.h < b.h || (a.h == b.h && a.l < b.l); }
__device__ __forceinline__ bool mf_dw_ge(mf_dw a, mf_dw b) { return a.h > b.h || (a.h == b.h && a.l >= b.l); }
__device__ __forceinline__ bool mf_dw_le(mf_dw a, mf_dw b) { return a.h < b.h || (a.h == b.h && a.l <= b.l); }
__device__ __forceinline__ bool mf_dw_eq(mf_dw a, mf_dw b) { return a.h == b.h && a.l == b.l; }
// A sum of logarithms as the logarithm of a running product (per thread):
// m * 2^e with m kept in [1, 2) by an exact power-of-two rescaling and the
// binary exponent e in an integer, so each factor costs one double-float
// product instead of a logarithm. A factor that is not positive (or NaN), or
// a product outside the FP32 normal range, makes m NaN for good; the
// thread's sum is then NaN, as a sum of the logs would be non-finite.
__device__ __forceinline__ void mf_dw_logprod(mf_dw& m, int& e, mf_dw p) {
  const mf_dw q = mf_dw_mul(m, p);
  const int ex = (int)((__float_as_uint(q.h) >> 23) & 0xffu);
  const float sc = __uint_as_float((unsigned)(254 - ex) << 23);  // 2^(127 - ex) for ex in [1, 253]
  const bool ok = p.h > 0.0f && ex > 0 && ex < 254;
  m = ok ? mf_dw_make(__fmul_rn(q.h, sc), __fmul_rn(q.l, sc)) : mf_dw_make(__int_as_float(0x7fc00000), 0.0f);
  e += ex - 127;
}
// log(m * 2^e) = log(m) + e ln2, ln2 as a double-float pair (e exact in FP32);
// a thread without factors (m = 1, e = 0) contributes exactly 0.
__device__ __forceinline__ mf_dw mf_dw_logprod_log(mf_dw m, int e, const float4* __restrict__ tab) {
  if (e == 0 && m.h == 1.0f && m.l == 0.0f) return mf_dw_make(0.0f, 0.0f);
  const mf_dw el = mf_dw_mul(mf_dw_make((float)e, 0.0f), mf_dw_make(MF_LN2_HI, MF_LN2_LO));
  return mf_dw_add(mf_dw_log(m, tab), el);
}
__device__ __forceinline__ mf_dw mf_dw_shfl_xor(mf_dw a, int o) {
  return mf_dw_make(__shfl_xor_sync(0xffffffffu, a.h, o), __shfl_xor_sync(0xffffffffu, a.l, o));
}
)CUDA";

// Bulk asynchronous global->shared copies completed on an mbarrier (sm_90+
// PTX: cp.async.bulk, mbarrier.*). Both addresses 16-byte aligned, sizes a
// multiple of 16 bytes.
const char* kBulkPrelude = R"CUDA(
__device__ __forceinline__ unsigned mf_smem_u32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mf_mbar_init(unsigned long long* b, unsigned cnt) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(mf_smem_u32(b)), "r"(cnt) : "memory");
}
__device__ __forceinline__ void mf_fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
__device__ __forceinline__ void mf_fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void mf_mbar_expect_tx(unsigned long long* b, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(mf_smem_u32(b)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void mf_bulk_g2s(void* dst, const void* src, unsigned bytes, unsigned long long* b) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
               ::"r"(mf_smem_u32(dst)), "l"(src), "r"(bytes), "r"(mf_smem_u32(b)) : "memory");
}
__device__ __forceinline__ unsigned mf_mbar_try_wait(unsigned long long* b, unsigned parity) {
  unsigned ok;
  asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
               : "=r"(ok) : "r"(mf_smem_u32(b)), "r"(parity) : "memory");
  return ok;
}
// Bounded wait: false after MF_SPIN_LIMIT unsuccessful polls.
#define MF_SPIN_LIMIT (1u << 22)
__device__ __forceinline__ bool mf_mbar_wait_bounded(unsigned long long* b, unsigned parity) {
  for (unsigned i = 0; i < MF_SPIN_LIMIT; i++)
    if (mf_mbar_try_wait(b, parity)) return true;
  return false;
}
)CUDA";

// 2^(j/64), j = 0..63, as double-float pairs {hi, lo} (hi the nearest float,
// lo the nearest float to the remainder), computed in 60-digit decimal
// arithmetic: the table of mf_dw_exp.
const char* const kExp2Table[64] = {
    "{0x1p+0f, 0x0p+0f}", "{0x1.02c9a4p+0f, -0x1.887fap-28f}",
    "{0x1.059b0ep+0f, -0x1.9d4f52p-25f}", "{0x1.087452p+0f, -0x1.e2990ep-26f}",
    "{0x1.0b5586p+0f, 0x1.9f3122p-25f}", "{0x1.0e3ec4p+0f, -0x1.a585ccp-25f}",
    "{0x1.11301ep+0f, -0x1.fdb496p-25f}", "{0x1.1429aap+0f, 0x1.d525bcp-25f}",
    "{0x1.172b84p+0f, -0x1.c15742p-27f}", "{0x1.1a35bep+0f, 0x1.6df96ep-25f}",
    "{0x1.1d4874p+0f, -0x1.d2e8cap-25f}", "{0x1.2063b8p+0f, 0x1.0c519ap-25f}",
    "{0x1.2387a6p+0f, 0x1.ceac48p-25f}", "{0x1.26b456p+0f, 0x1.789f38p-26f}",
    "{0x1.29e9ep+0f, -0x1.5c0424p-25f}", "{0x1.2d285ap+0f, 0x1.b900c2p-26f}",
    "{0x1.306fep+0f, 0x1.4636e2p-25f}", "{0x1.33c08cp+0f, -0x1.b37d2p-25f}",
    "{0x1.371a74p+0f, -0x1.18aac6p-25f}", "{0x1.3a7db4p+0f, -0x1.634c02p-25f}",
    "{0x1.3dea64p+0f, 0x1.824684p-25f}", "{0x1.4160a2p+0f, 0x1.f72e2ap-28f}",
    "{0x1.44e086p+0f, 0x1.8624b4p-30f}", "{0x1.486a2cp+0f, -0x1.47d866p-25f}",
    "{0x1.4bfdaep+0f, -0x1.593abcp-25f}", "{0x1.4f9b28p+0f, -0x1.2c5a6cp-25f}",
    "{0x1.5342b6p+0f, -0x1.2c561p-25f}", "{0x1.56f474p+0f, -0x1.295b04p-25f}",
    "{0x1.5ab07ep+0f, -0x1.5bd5ecp-27f}", "{0x1.5e76f2p+0f, -0x1.4a5bd6p-25f}",
    "{0x1.6247ecp+0f, -0x1.f8b55p-25f}", "{0x1.662388p+0f, 0x1.2a9112p-27f}",
    "{0x1.6a09e6p+0f, 0x1.9fcef4p-26f}", "{0x1.6dfb24p+0f, -0x1.cd72e8p-27f}",
    "{0x1.71f75ep+0f, 0x1.1d8beep-25f}", "{0x1.75feb6p+0f, -0x1.37b306p-25f}",
    "{0x1.7a1148p+0f, -0x1.829fdp-25f}", "{0x1.7e2f34p+0f, -0x1.261634p-25f}",
    "{0x1.82589ap+0f, -0x1.accc7cp-26f}", "{0x1.868d9ap+0f, -0x1.2edb44p-26f}",
    "{0x1.8ace54p+0f, 0x1.15506ep-27f}", "{0x1.8f1aeap+0f, -0x1.baa232p-26f}",
    "{0x1.93737cp+0f, -0x1.e64744p-25f}", "{0x1.97d82ap+0f, -0x1.0d8d84p-31f}",
    "{0x1.9c4918p+0f, 0x1.51f848p-27f}", "{0x1.a0c668p+0f, -0x1.2886a6p-26f}",
    "{0x1.a5503cp+0f, -0x1.b83b54p-25f}", "{0x1.a9e6b6p+0f, -0x1.50c048p-25f}",
    "{0x1.ae89fap+0f, -0x1.a94b14p-26f}", "{0x1.b33a2cp+0f, -0x1.ec3a82p-26f}",
    "{0x1.b7f77p+0f, -0x1.a09438p-25f}", "{0x1.bcc1eap+0f, -0x1.f687c6p-25f}",
    "{0x1.c199bep+0f, -0x1.3d56b2p-27f}", "{0x1.c67f12p+0f, 0x1.cafa2ap-25f}",
    "{0x1.cb720ep+0f, -0x1.8837ccp-27f}", "{0x1.d072d4p+0f, 0x1.40f13p-25f}",
    "{0x1.d5818ep+0f, -0x1.822dbcp-27f}", "{0x1.da9e6p+0f, 0x1.ed9942p-27f}",
    "{0x1.dfc974p+0f, -0x1.908c94p-25f}", "{0x1.e502eep+0f, 0x1.e2cffep-26f}",
    "{0x1.ea4afap+0f, 0x1.52486cp-27f}", "{0x1.efa1bep+0f, 0x1.cc2b44p-25f}",
    "{0x1.f50766p+0f, -0x1.246ebp-26f}", "{0x1.fa7c18p+0f, 0x1.9e90d8p-28f}"};

// The 128-entry table of mf_dw_log: for c_j = 1 + (2j+1)/256,
// {hi(ln c_j), lo(ln c_j), 1/c_j, c_j} as exact float literals; and the
// 64-entry table of mf_dw_exp.
std::string dw_log_table() {
  std::ostringstream o;
  {
    const double ln2 = std::log(2.0);
    const float hi = float(ln2), lo = float(ln2 - double(hi));
    char b[160];
    std::snprintf(b, sizeof b, "#define MF_LN2_HI %af\n#define MF_LN2_LO %af\n", double(hi), double(lo));
    o << b;
  }
  o << "__device__ const float4 mf_dw_logtab_g[128] = {\n";
  for (int j = 0; j < 128; j++) {
    const double c = 1.0 + (2.0 * j + 1.0) / 256.0;
    const double L = std::log(c);
    const float lh = float(L);
    const float ll = float(L - double(lh));
    const float ic = float(1.0 / c);
    char b[200];
    std::snprintf(b, sizeof b, "  {%af, %af, %af, %af},\n", double(lh), double(ll), double(ic), c);
    o << b;
  }
  o << "};\n";
  o << "__device__ const float2 mf_dw_exptab_g[64] = {\n";
  for (const char* row : kExp2Table) o << "  " << row << ",\n";
  o << "};\n";
  return o.str();
}

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
                    const GenerateSpec* gen, bool native_f64, int vec_req, int block_req, bool f32_arith,
                    bool direct_loads, int stages_req, const std::vector<std::string>& param_defs) {
  std::vector<std::string> in_names = inputs;
  if (kind == Kind::Generate) {
    if (!gen) throw std::runtime_error("generate kernel without generate spec");
    in_names = gen->dims;
  }
  Dag dag(in_names, params);
  std::vector<int> roots0;
  for (auto& e : exprs) roots0.push_back(dag.parse(e));
  std::vector<int> source_inputs;
  {
    const auto& n0 = dag.nodes();
    const auto l0 = reachable(n0, roots0);
    std::set<int> u;
    for (size_t i = 0; i < n0.size(); i++)
      if (l0[i] && n0[i].op == Op::Input) u.insert(n0[i].index);
    source_inputs.assign(u.begin(), u.end());
  }
  const bool st32 = (elem == Elem::F32);
  // REDUCE kernels read prepared columns when that pays: double-float
  // kernels always (FP64 values stored pre-split as float pairs, so the event
  // loop does no splitting), FP32 and native FP64 kernels when linearly
  // dependent columns fold. FP32-over-FP64 kernels read the source columns.
  FoldResult fold;
  int prep = LoweredKernel::PrepNone;
  if (kind == Kind::Reduce && !f32_arith) {
    fold = fold_columns(dag, roots0, param_defs);
    const bool dw = !st32 && !native_f64;
    if (fold.rewritten && (dw || fold.folded))
      prep = dw ? LoweredKernel::PrepPair : st32 ? LoweredKernel::PrepF32 : LoweredKernel::PrepF64;
  }
  const Dag& G = prep ? *fold.dag : dag;
  const std::vector<int>& roots = prep ? fold.roots : roots0;
  const auto& ns = G.nodes();
  auto live = reachable(ns, roots);

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
  if (kind == Kind::Reduce) {
    out.pipelined = !direct_loads;
    // double-float bodies: one event per thread per iteration, 512 threads
    // (measured fastest on GB300 for the K*mumu gradient kernel)
    const bool dw_default = !st32 && !native_f64 && !f32_arith;
    if (dw_default) {
      // two events per thread (one 16-byte load per prepared column) for
      // gradient-sized kernels, measured fastest on GB300 for the K*mumu
      // gradient; many-output kernels (Hessians) take one event per thread so
      // their accumulators stay in registers
      out.vec = (!out.pipelined && exprs.size() <= 16) ? 2 : 1;
    }
    // FP32 Hessian-sized kernels: one event per thread as well (measured on
    // GB300: K*mumu P-wave Hessian 12.1 vs 13.4 us at four events per thread,
    // S+P-wave Hessian, 105 outputs, 58.7 vs 70.6 us per 1M events)
    if (st32 && !out.pipelined && exprs.size() > 16) out.vec = 1;
    if (vec_req == 1 || vec_req == 2 || (vec_req == 4 && st32)) out.vec = vec_req;
    if (block_req >= 64 && block_req <= 1024 && block_req % 32 == 0) out.block = block_req;
    // bulk-copy pipeline: shared-memory stages; direct loads: loop unroll
    // factor (1 = none). Gradient-sized kernels (at most 16 outputs) unroll
    // twice by default: with batched evaluations overlapping, the next
    // iteration's loads issued before this one's arithmetic measured fastest
    // on GB300 (K*mumu gradient 11.4 vs 12.1 us per 1M-event evaluation in
    // double-float, 5.9 vs 6.5 us in FP32); Hessian-sized kernels keep their
    // accumulators in registers with one iteration in flight.
    // Many-output double-float kernels (the S+P-wave Hessian: 105 outputs)
    // cannot keep every per-thread partial in registers: the outputs beyond
    // acc_reg keep theirs in shared memory instead (each thread its own
    // column, 8 bytes per output), in blocks of 64 threads unless a block
    // size is asked for, so that the kernel neither spills nor reads the
    // dataset more than once (S+P-wave Hessian at 1M events, batched: 157 us,
    // against 301 us spilling and 189 us as three register-only kernels).
    // FP32 partials are cheap enough that the shared-memory traffic costs more
    // than it saves (85 us against 49 us as three kernels): not for FP32.
    if (!out.pipelined && int(exprs.size()) > kAccRegMax && dw_default) {
      if (block_req == 0) out.block = 64;
      const int room = int(kAccSmemBytes / (8 * size_t(out.block)));
      out.acc_reg = std::max(int(exprs.size()) - room, kAccRegMin);
    }
    if (out.pipelined)
      out.stages = stages_req >= 2 && stages_req <= 8 ? stages_req : (dw_default ? 3 : 4);
    else
      out.stages = stages_req >= 1 && stages_req <= 4 ? stages_req
                                                     : (!native_f64 && exprs.size() <= 16 ? 2 : 1);
    out.tile = out.block * out.vec;
  }
  const int V = out.vec;
  const int M = int(exprs.size());
  const int NP = std::max<int>(1, int(params.size()));

  std::set<int> used;
  for (size_t i = 0; i < ns.size(); i++)
    if (live[i] && ns[i].op == Op::Input) used.insert(ns[i].index);
  out.used_inputs.assign(used.begin(), used.end());
  out.source_inputs = source_inputs;
  out.prep = prep;
  if (prep) out.prep_cols = fold.cols;
  const bool pair = prep == LoweredKernel::PrepPair;
  if (pair && V != 1 && V != 2) throw std::runtime_error("double-float kernels take 1 or 2 events per thread");

  std::ostringstream s;
  s << "// MoreFit CUDA backend: generated kernel '" << name << "' (" << (kind == Kind::Reduce ? "reduce"
                                                                          : kind == Kind::Store ? "store"
                                                                                                : "generate")
    << ", " << ST << " storage, "
    << (kind == Kind::Reduce && !st32 && !native_f64 ? std::string("double-float") : AT) << " arithmetic)\n";
  if (prep) {
    s << "// reads " << fold.cols.size() << " prepared columns (" << (pair ? "FP64 as float pairs" : st32 ? "FP32" : "FP64")
      << ") derived from " << fold.source_columns << " source columns:\n";
    for (size_t m = 0; m < fold.cols.size(); m++) {
      s << "//   y" << m << " =";
      for (auto& [col, c] : fold.cols[m]) s << " + " << c << "*" << in_names[col];
      s << "\n";
    }
  }
  s << "// outputs:\n";
  for (size_t j = 0; j < exprs.size(); j++) s << "//   [" << j << "] " << exprs[j].substr(0, 160) << "\n";
  s << kPrelude;
  if (out.acc_reg <= 0 || out.acc_reg > M) out.acc_reg = M;
  const int NREG = out.acc_reg;
  s << "#define MF_BLOCK " << out.block << "\n#define MF_NOUT " << M << "\n#define MF_NPAR " << NP << "\n";
  // per-thread partials of outputs [0, MF_NREG) in registers, the rest in shared memory
  s << "#define MF_NREG " << NREG << "\n";
  // launch bounds of the event-loop entries
  s << "#define MF_BOUNDS __launch_bounds__(MF_BLOCK)\n";
  // partial blocks each last-block thread loads per round (bounded register use)
  // combine of block partial rows: MF_CC outputs at a time, MF_Q rows of each in flight per thread
  // (up to 16 outputs and up to four rows of each, about 32 values per thread
  // in flight: a grid of two blocks per SM leaves each thread of the last
  // block one or two rows, so its loads go out in one round; many-output
  // kernels, whose grids of small blocks leave thousands of partial rows, take
  // eight outputs and four rows at a time)
  const int cc = M > kAccRegMax ? 8 : std::min(M, 16);
  s << "#define MF_CC " << cc << "\n";
  s << "#define MF_Q " << (M > kAccRegMax ? 4 : std::max(1, std::min(4, 32 / cc))) << "\n";
  // outputs per block-reduction chunk (one warp each)
  s << "#define MF_RC " << std::max(1, std::min(8, out.block / 32)) << "\n";
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

  if (kind == Kind::Reduce || (kind == Kind::Store && !native_f64)) {
    // Arithmetic of the per-event body: FP32 (mixed precision), FP64, or
    // double-float on FP32 pairs (the default for FP64 storage, and for
    // STORE kernels unless native FP64 is asked for).
    // F32S: FP64 storage, FP32 arithmetic, except that a sum or difference of
    // an input column and a parameter-only value is formed in FP64 before it
    // is rounded (keeps m - mu exact for observables with a large offset).
    enum class Ar { F32, F64, DW, F32S } ar =
        kind == Kind::Store ? Ar::DW : st32 ? Ar::F32 : (f32_arith ? Ar::F32S : (native_f64 ? Ar::F64 : Ar::DW));
    auto is_leafish = [&](int k) {
      const Op o = ns[k].op;
      return o == Op::Input || ns[k].uniform;
    };
    // per-event nodes evaluated in FP64 under F32S
    std::vector<char> dnode(ns.size(), 0);
    if (ar == Ar::F32S)
      for (size_t i = 0; i < ns.size(); i++) {
        const Node& n = ns[i];
        if (!live[i] || n.uniform || (n.op != Op::Add && n.op != Op::Sub)) continue;
        if (is_leafish(n.a) && is_leafish(n.b) && (ns[n.a].op == Op::Input || ns[n.b].op == Op::Input)) dnode[i] = 1;
      }
    // Double-float exp and pow (table-driven, FP32 pipe) in REDUCE kernels,
    // whose non-finite sums are re-evaluated in native FP64 by the runtime;
    // STORE kernels write columns and keep FP64 exp / pow (full FP64 range).
    const bool dw_exp = kind == Kind::Reduce;
    bool has_log = false, has_exp = false;
    for (size_t i = 0; i < ns.size(); i++) {
      if (!live[i] || ns[i].uniform) continue;
      if (ns[i].op == Op::Log || (dw_exp && ns[i].op == Op::Pow)) has_log = true;
      if (dw_exp && (ns[i].op == Op::Exp || ns[i].op == Op::Pow)) has_exp = true;
    }
    // The double-float library is always present: every cross-thread sum
    // (warp, block, grid) runs in double-float on the FP32 pipe.
    s << dw_log_table() << kDwPrelude << (kind == Kind::Reduce ? kBulkPrelude : "");
    // ---- leaves and statements of the per-event body ----
    auto eref = [&](int id) -> std::string {
      const Node& n = ns[id];
      if (ar == Ar::F32S) {  // float view of any node
        if (n.op == Op::Const) return fmt_const(n.value, true);
        if (n.op == Op::Input) return "(float)x" + std::to_string(n.index);
        if (n.op == Op::Param) return "pf" + std::to_string(n.index);
        if (n.uniform) return "uf" + std::to_string(id);
        if (dnode[id]) return "(float)e" + std::to_string(id);
        return "e" + std::to_string(id);
      }
      if (n.op == Op::Const) {
        if (ar == Ar::F32) return fmt_const(n.value, true);
        if (ar == Ar::F64) return fmt_const(n.value, false);
        const float h = float(n.value);
        const float l = float(n.value - double(h));
        char b[96];
        std::snprintf(b, sizeof b, "mf_dw_make(%af, %af)", double(h), double(l));
        return b;
      }
      if (n.op == Op::Input) return "x" + std::to_string(n.index);
      const std::string sfx = ar == Ar::F32 ? "f" : ar == Ar::DW ? "w" : "";
      if (n.op == Op::Param) return "p" + sfx + std::to_string(n.index);
      if (n.uniform) return "u" + sfx + std::to_string(id);
      return "e" + std::to_string(id);
    };
    auto dref = [&](int k) -> std::string {  // FP64 view of an input / uniform / constant (F32S only)
      const Node& n = ns[k];
      if (n.op == Op::Const) return fmt_const(n.value, false);
      if (n.op == Op::Input) return "x" + std::to_string(n.index);
      if (n.op == Op::Param) return "p" + std::to_string(n.index);
      return "u" + std::to_string(k);
    };
    // operands of which both sin and cos are live per-event values: node -> (sin node, cos node)
    std::map<int, std::pair<int, int>> sincos_pair;
    if (ar == Ar::DW) {
      std::map<int, int> sin_of, cos_of;
      for (size_t i = 0; i < ns.size(); i++) {
        if (!live[i] || ns[i].uniform) continue;
        if (ns[i].op == Op::Sin) sin_of[ns[i].a] = int(i);
        if (ns[i].op == Op::Cos) cos_of[ns[i].a] = int(i);
      }
      for (auto& [a, si] : sin_of) {
        auto c = cos_of.find(a);
        if (c != cos_of.end()) sincos_pair[a] = {si, c->second};
      }
    }
    // Double-float REDUCE bodies: sums of (value x parameter-only factor)
    // terms become compensated dot products, and an output that is a product
    // used nowhere else is multiplied straight into its accumulator.
    std::vector<int> uses(ns.size(), 0), consumer(ns.size(), -1);
    std::vector<char> skip(ns.size(), 0);
    std::map<int, std::vector<std::pair<int, int>>> chains;  // chain root -> its terms (a, b)
    std::vector<std::pair<int, int>> fused(roots.size(), {-1, -1});
    std::vector<int> logprod(roots.size(), -1);  // output j = log(node) summed as a running product
    // ... plus (or minus) a parameter-only value per event (the normalisation
    // term of logprob_normalised, pdf.hh:103-106): log(x) + u or log(x) - u
    std::vector<int> logadd(roots.size(), -1), logsign(roots.size(), 0), lognode(roots.size(), -1);
    // Double-float outputs x + u or x - u with u parameter-only (the
    // normalisation terms of Hessian outputs): x is accumulated and the
    // thread's event count times u added once, before the block reduction.
    std::vector<int> addu(roots.size(), -1), addsign(roots.size(), 0), accnode(roots);
    // FP32 REDUCE bodies (mixed precision) whose only output is the logarithm
    // of a dot product of per-event values with parameter-only factors (the
    // fitter's NLL kernel for a density linear in its prepared columns): that
    // dot product is kept as a compensated double-float value and its
    // logarithm summed as a double-float running product, so the NLL carries
    // no per-event FP32 rounding. Minuit2 takes function values from this
    // kernel (minuit2_grad_fcn::DoEval, fitter.hh:131-136) and compares them
    // in its line searches, which FP32 rounding noise of ~1e-7 per event
    // (1e-4 in the NLL of 1M events) would disturb. Kernels with gradient
    // outputs keep plain FP32 arithmetic: Minuit2 discards their NLL value
    // (fitter.hh:138-144), and their cost per event stays at the FP32 rate.
    std::set<int> f32_dw_chain;  // chain roots evaluated in double-float under F32
    if ((ar == Ar::DW || ar == Ar::F32) && kind == Kind::Reduce) {
      for (size_t i = 0; i < ns.size(); i++) {
        if (!live[i] || ns[i].uniform || ns[i].op == Op::Input) continue;
        for (int c : {ns[i].a, ns[i].b, ns[i].c})
          if (c >= 0) {
            uses[c]++;
            consumer[c] = int(i);
          }
      }
      for (int r : roots) {
        uses[r]++;
        consumer[r] = -1;
      }
      auto is_term = [&](int k) {
        const Node& n = ns[k];
        return n.op == Op::Mul && !n.uniform && uses[k] == 1 && (ns[n.a].uniform || ns[n.b].uniform);
      };
      std::vector<char> chain(ns.size(), 0);
      for (size_t i = 0; i < ns.size(); i++) {
        const Node& n = ns[i];
        if (!live[i] || n.uniform || n.op != Op::Add) continue;
        auto part = [&](int c) { return is_term(c) || (chain[c] && uses[c] == 1); };
        if (part(n.a) && part(n.b)) chain[i] = 1;
      }
      std::function<void(int, std::vector<std::pair<int, int>>&)> collect = [&](int k, auto& terms) {
        if (chain[k]) {
          collect(ns[k].a, terms);
          collect(ns[k].b, terms);
        } else {
          terms.push_back({ns[k].a, ns[k].b});
        }
      };
      // Output r as log(x) [+ or - u]: the Log node (used only there), u, sign.
      auto log_form = [&](int r, int& lg, int& u, int& sign) {
        lg = -1;
        u = -1;
        sign = 0;
        const Node& n = ns[r];
        if (n.uniform || uses[r] != 1) return false;
        auto is_log = [&](int k) { return ns[k].op == Op::Log && !ns[k].uniform && uses[k] == 1; };
        if (is_log(r)) {
          lg = r;
          return true;
        }
        if (n.op == Op::Add || n.op == Op::Sub) {
          if (is_log(n.a) && ns[n.b].uniform) {
            lg = n.a;
            u = n.b;
            sign = n.op == Op::Add ? 1 : -1;
            return true;
          }
          if (n.op == Op::Add && is_log(n.b) && ns[n.a].uniform) {
            lg = n.b;
            u = n.a;
            sign = 1;
            return true;
          }
        }
        return false;
      };
      if (ar == Ar::F32) {
        // only the chain that is the argument of the single output's logarithm
        std::set<int> wanted;
        for (int r : roots) {
          int lg, u, sg;
          if (M == 1 && log_form(r, lg, u, sg) && chain[ns[lg].a]) wanted.insert(ns[lg].a);
        }
        for (size_t i = 0; i < ns.size(); i++)
          if (chain[i] && !wanted.count(int(i))) {
            // keep chain marks only below a wanted root
            bool below = false;
            for (int c = consumer[i]; c >= 0 && !below; c = (uses[c] == 1 && chain[c]) ? consumer[c] : -1)
              below = wanted.count(c) > 0;
            if (!below) chain[i] = 0;
          }
        f32_dw_chain = wanted;
      }
      for (size_t i = 0; i < ns.size(); i++) {
        if (!chain[i]) continue;
        const bool absorbed = uses[i] == 1 && consumer[i] >= 0 && chain[consumer[i]];
        if (absorbed) continue;
        std::vector<std::pair<int, int>> terms;
        collect(int(i), terms);
        chains[int(i)] = terms;
        // every node of the chain below its root is folded into the root's statement
        std::function<void(int)> mark = [&](int k) {
          if (k != int(i)) skip[k] = 1;
          if (chain[k]) {
            mark(ns[k].a);
            mark(ns[k].b);
          }
        };
        mark(int(i));
      }
      for (size_t j = 0; j < roots.size(); j++) {
        const int r = roots[j];
        const Node& n = ns[r];
        int lg = -1, u = -1, sg = 0;
        const bool lf = !skip[r] && log_form(r, lg, u, sg);
        if (ar == Ar::F32) {
          if (lf && f32_dw_chain.count(ns[lg].a)) {
            logprod[j] = ns[lg].a;
            logadd[j] = u;
            logsign[j] = sg;
            lognode[j] = lg;
            skip[r] = 1;
            skip[lg] = 1;
          }
          continue;
        }
        if (n.op == Op::Mul && !n.uniform && uses[r] == 1 && !chains.count(r) && !skip[r]) {
          fused[j] = {n.a, n.b};
          skip[r] = 1;
        }
        if (ar == Ar::DW && !lf && !skip[r] && uses[r] == 1 && !n.uniform && (n.op == Op::Add || n.op == Op::Sub)) {
          int x = -1, u = -1, sg = 0;
          if (ns[n.b].uniform && !ns[n.a].uniform) {
            x = n.a;
            u = n.b;
            sg = n.op == Op::Add ? 1 : -1;
          } else if (n.op == Op::Add && ns[n.a].uniform && !ns[n.b].uniform) {
            x = n.b;
            u = n.a;
            sg = 1;
          }
          if (x >= 0 && !skip[x] && !chains.count(x)) {
            addu[j] = u;
            addsign[j] = sg;
            accnode[j] = x;
            skip[r] = 1;
            const Node& xn = ns[x];
            if (xn.op == Op::Mul && uses[x] == 1 && ns[x].op != Op::Input) {
              fused[j] = {xn.a, xn.b};
              skip[x] = 1;
            }
          }
        }
        // an output that is the logarithm of a per-event value (plus or minus a
        // parameter-only value), used nowhere else: sum of logs = log of the
        // product (one multiply per event), plus the event count times u
        if (lf && !skip[r]) {
          logprod[j] = ns[lg].a;
          logadd[j] = u;
          logsign[j] = sg;
          lognode[j] = lg;
          skip[r] = 1;
          skip[lg] = 1;
        }
      }
    }
    bool has_addu = false;
    for (int u : addu) has_addu = has_addu || u >= 0;
    auto estmt = [&](int id) -> std::string {
      const Node& n = ns[id];
      if (ar == Ar::F32S && dnode[id])
        return "const double e" + std::to_string(id) + " = " + dref(n.a) + (n.op == Op::Add ? " + " : " - ") + dref(n.b) +
               ";";
      const std::string T = ar == Ar::F32 || ar == Ar::F32S ? "float" : ar == Ar::F64 ? "double" : "mf_dw";
      const std::string lhs = "const " + std::string(n.op == Op::Cmp ? "bool" : T) + " e" + std::to_string(id) + " = ";
      const std::string A = n.a >= 0 ? eref(n.a) : "", B = n.b >= 0 ? eref(n.b) : "", Cc = n.c >= 0 ? eref(n.c) : "";
      if (ar == Ar::F32 && skip[id]) return "";
      if (ar == Ar::F32 && chains.count(id)) {
        // terms value x factor, the parameter-only factor as a double-float
        // pair (so that the sum follows the FP64 parameters smoothly)
        const std::string e = "e" + std::to_string(id);
        const auto& terms = chains.at(id);
        std::string c = "mf_dw w" + e + "; { mf_dw t_;";
        for (size_t q = 0; q < terms.size(); q++) {
          const bool a_uni = ns[terms[q].first].uniform;
          const int u = a_uni ? terms[q].first : terms[q].second, v = a_uni ? terms[q].second : terms[q].first;
          std::string cw;
          if (ns[u].op == Op::Const) {
            const float h = float(ns[u].value);
            char b[96];
            std::snprintf(b, sizeof b, "mf_dw_make(%af, %af)", double(h), double(float(ns[u].value - double(h))));
            cw = b;
          } else {
            cw = "uw" + std::to_string(u);
          }
          c += q == 0 ? " t_ = mf_dw_prodfw(" + eref(v) + ", " + cw + ");"
                      : " mf_dw_acc_mulfw(t_, " + eref(v) + ", " + cw + ");";
        }
        return c + " w" + e + " = mf_dw_renorm(t_); } const float " + e + " = w" + e + ".h;";
      }
      if (ar != Ar::DW) {
        const bool f = ar == Ar::F32 || ar == Ar::F32S;
        switch (n.op) {
          case Op::Add: return lhs + A + " + " + B + ";";
          case Op::Sub: return lhs + A + " - " + B + ";";
          case Op::Mul: return lhs + A + " * " + B + ";";
          case Op::Div: return lhs + A + " / " + B + ";";
          case Op::Neg: return lhs + "-" + A + ";";
          case Op::Rcp: return lhs + fn_name(Op::Rcp, f) + "(" + A + ");";
          case Op::Pow: return lhs + fn_name(Op::Pow, f) + "(" + A + ", " + B + ");";
          case Op::Cmp: return lhs + "(" + A + " " + cmp_str(n.cmp) + " " + B + ");";
          case Op::Select: return lhs + "(" + A + " ? " + B + " : " + Cc + ");";
          default:
            if (is_unary_fn(n.op)) return lhs + fn_name(n.op, f) + "(" + A + ");";
        }
        throw std::runtime_error("emit: unexpected node");
      }
      auto D = [](const std::string& v) { return "mf_dw_to_double(" + v + ")"; };
      if (skip[id]) return "";
      auto ch = chains.find(id);
      if (ch != chains.end()) {
        std::string c = "mf_dw e" + std::to_string(id) + "; { mf_dw t_ = mf_dw_make(0.0f, 0.0f);";
        for (auto& [ta, tb] : ch->second) c += " mf_dw_acc_mul(t_, " + eref(ta) + ", " + eref(tb) + ");";
        return c + " e" + std::to_string(id) + " = mf_dw_renorm(t_); }";
      }
      switch (n.op) {
        case Op::Add: return lhs + "mf_dw_add(" + A + ", " + B + ");";
        case Op::Sub: return lhs + "mf_dw_sub(" + A + ", " + B + ");";
        case Op::Mul: return lhs + "mf_dw_mul(" + A + ", " + B + ");";
        case Op::Div: return lhs + "mf_dw_mul(" + A + ", mf_dw_rcp(" + B + "));";
        case Op::Neg: return lhs + "mf_dw_neg(" + A + ");";
        case Op::Rcp: return lhs + "mf_dw_rcp(" + A + ");";
        case Op::Log: return lhs + "mf_dw_log(" + A + ", mf_logtab);";
        case Op::Sqrt: return lhs + "mf_dw_sqrt(" + A + ");";
        case Op::Sin:
        case Op::Cos: {
          // sin and cos of the same operand share one reduction and both polynomials
          auto it = sincos_pair.find(n.a);
          if (it == sincos_pair.end()) return lhs + (n.op == Op::Sin ? "mf_dw_sin(" : "mf_dw_cos(") + A + ");";
          const int first = std::min(it->second.first, it->second.second);
          if (id != first) return "";  // defined with the first of the two
          const std::string sn = "e" + std::to_string(it->second.first), cn = "e" + std::to_string(it->second.second);
          return "mf_dw " + sn + ", " + cn + "; mf_dw_sincos(" + A + ", &" + sn + ", &" + cn + ");";
        }
        case Op::Pow:
          if (dw_exp) return lhs + "mf_dw_pow(" + A + ", " + B + ", mf_logtab, mf_exptab);";
          return lhs + "mf_dw_from_double(pow(" + D(A) + ", " + D(B) + "));";
        case Op::Exp:
          if (dw_exp) return lhs + "mf_dw_exp(" + A + ", mf_exptab);";
          return lhs + "mf_dw_from_double(exp(" + D(A) + "));";
        case Op::Cmp:
          switch (n.cmp) {
            case CmpOp::Gt: return lhs + "mf_dw_gt(" + A + ", " + B + ");";
            case CmpOp::Lt: return lhs + "mf_dw_lt(" + A + ", " + B + ");";
            case CmpOp::Ge: return lhs + "mf_dw_ge(" + A + ", " + B + ");";
            case CmpOp::Le: return lhs + "mf_dw_le(" + A + ", " + B + ");";
            case CmpOp::Eq: return lhs + "mf_dw_eq(" + A + ", " + B + ");";
            case CmpOp::Ne: return lhs + "!mf_dw_eq(" + A + ", " + B + ");";
          }
          break;
        case Op::Select: return lhs + "(" + A + " ? " + B + " : " + Cc + ");";
        default:
          if (is_unary_fn(n.op)) return lhs + "mf_dw_from_double(" + fn_name(n.op, false) + "(" + D(A) + "));";
      }
      throw std::runtime_error("emit: unexpected node");
    };
    if (kind == Kind::Store) {
      // Event-only precompute in double-float: inputs split with rounding
      // and outputs joined by integer operations (the FP64 pipe, 1/64 of the
      // FP32 rate on GB300, is not used per event), parameter-only values
      // evaluated in FP64 once per thread.
      std::set<int> uni;
      for (size_t i = 0; i < ns.size(); i++) {
        if (!live[i] || ns[i].uniform || ns[i].op == Op::Input) continue;
        for (int c : {ns[i].a, ns[i].b, ns[i].c})
          if (c >= 0 && ns[c].uniform && ns[c].op != Op::Const) uni.insert(c);
      }
      for (int r : roots)
        if (ns[r].uniform && ns[r].op != Op::Const) uni.insert(r);
      s << "extern \"C\" __global__ void __launch_bounds__(MF_BLOCK) " << out.entry << "(const " << ST
        << "* __restrict__ data, mf_u64 stride, mf_u64 n, mf_par P, " << ST
        << "* __restrict__ outp, mf_u64 out_stride) {\n";
      if (has_log)
        s << "  __shared__ float4 mf_logtab[128];\n"
          << "  for (int q = threadIdx.x; q < 128; q += MF_BLOCK) mf_logtab[q] = mf_dw_logtab_g[q];\n"
          << "  __syncthreads();\n";
      emit_params_and_uniform(s, "P.v");
      for (int k : uni)
        s << "  const mf_dw " << eref(k) << " = mf_dw_from_double(" << dref(k) << ");\n";
      s << "  const mf_u64 step = (mf_u64)gridDim.x * MF_BLOCK;\n";
      s << "  for (mf_u64 i = (mf_u64)blockIdx.x * MF_BLOCK + threadIdx.x; i < n; i += step) {\n";
      for (int k : out.used_inputs)
        s << "    const mf_dw x" << k << " = mf_dw_split_rn((double)data[(mf_u64)" << k << " * stride + i]);\n";
      for (size_t i = 0; i < ns.size(); i++) {
        if (!live[i] || ns[i].uniform || ns[i].op == Op::Input) continue;
        const std::string st = estmt(int(i));
        if (!st.empty()) s << "    " << st << "\n";
      }
      for (int j = 0; j < M; j++) {
        const Node& r = ns[roots[j]];
        if (r.op == Op::Input)  // a copied column stays bit-exact
          s << "    outp[(mf_u64)" << j << " * out_stride + i] = data[(mf_u64)" << r.index << " * stride + i];\n";
        else if (st32)  // h + l rounded once
          s << "    { const mf_dw o = " << eref(roots[j]) << "; outp[(mf_u64)" << j
            << " * out_stride + i] = __fadd_rn(o.h, o.l); }\n";
        else
          s << "    outp[(mf_u64)" << j << " * out_stride + i] = mf_dw_to_double_bits(" << eref(roots[j]) << ");\n";
      }
      s << "  }\n}\n";
      out.source = s.str();
      return out;
    }
    // Uniform (parameter-only) values referenced by the per-event body or by an output.
    std::set<int> uni_used;
    auto note_uniform = [&](int k) {
      if (k >= 0 && ns[k].uniform && ns[k].op != Op::Const) uni_used.insert(k);
    };
    for (size_t i = 0; i < ns.size(); i++) {
      if (!live[i] || ns[i].uniform || ns[i].op == Op::Input || dnode[i]) continue;
      note_uniform(ns[i].a);
      note_uniform(ns[i].b);
      note_uniform(ns[i].c);
    }
    for (int r : roots) note_uniform(r);
    // Parameter-only values: evaluated once per launch on the host and passed
    // pre-rounded in the argument struct (no FP64 work in the kernel, where
    // FP64 issues at 1/64 of the FP32 rate).
    std::map<int, std::string> slot_names;  // node -> C name in the body
    {
      std::vector<UniformSlot> slots;
      int nd = 0, nf = 0;
      auto add_slot = [&](int k, int kind) {
        UniformSlot sl{k, kind, kind == UniformSlot::Double ? nd : nf};
        if (kind == UniformSlot::Double)
          nd++;
        else
          nf += kind == UniformSlot::DwPair ? 2 : 1;
        slots.push_back(sl);
      };
      std::set<int> dslots;  // nodes needed as doubles
      if (ar == Ar::F64) dslots = uni_used;
      if (ar == Ar::F32S)
        for (size_t i = 0; i < ns.size(); i++)
          if (dnode[i]) {
            if (ns[ns[i].a].uniform && ns[ns[i].a].op != Op::Const) dslots.insert(ns[i].a);
            if (ns[ns[i].b].uniform && ns[ns[i].b].op != Op::Const) dslots.insert(ns[i].b);
          }
      for (int k : dslots) {
        add_slot(k, UniformSlot::Double);
        slot_names[k] = ns[k].op == Op::Param ? "p" + std::to_string(ns[k].index) : "u" + std::to_string(k);
      }
      if (ar != Ar::F64)
        for (int k : uni_used)
          add_slot(k, ns[k].op == Op::Cmp ? UniformSlot::Bool : ar == Ar::DW ? UniformSlot::DwPair : UniformSlot::Float);
      if (ar == Ar::F32) {  // double-float factors of the compensated NLL dot product ("uw<node>")
        std::set<int> fac;
        for (auto& [root, terms] : chains)
          for (auto& [ta, tb] : terms) {
            const int u = ns[ta].uniform ? ta : tb;
            if (ns[u].op != Op::Const) fac.insert(u);
          }
        for (int j = 0; j < M; j++)
          if (logadd[j] >= 0 && ns[logadd[j]].op != Op::Const) fac.insert(logadd[j]);
        for (int k : fac) {
          add_slot(k, UniformSlot::DwPair);
          slot_names[k] = "uw" + std::to_string(k);
        }
      }
      out.host_args = true;
      out.nodes = ns;
      out.slots = slots;
      {
        // nodes reachable from the slots, in id order: a node's operands
        // always have smaller ids (hash-consed construction)
        std::vector<char> need(ns.size(), 0);
        for (const auto& sl : slots) need[sl.node] = 1;
        for (size_t i = ns.size(); i-- > 0;) {
          if (!need[i]) continue;
          for (int c : {ns[i].a, ns[i].b, ns[i].c}) {
            if (c >= int(i)) throw std::runtime_error("lowering: operand after its node");
            if (c >= 0) need[c] = 1;
          }
        }
        for (size_t i = 0; i < ns.size(); i++)
          if (need[i]) out.eval_order.push_back(int(i));
      }
      out.nd = std::max(1, nd);
      out.nf = std::max(1, nf);
    }
    auto prologue = [&](std::ostringstream& o, const std::string& P) {
      for (const auto& sl : out.slots) {
        const int k = sl.node;
        const std::string off = std::to_string(sl.offset);
        switch (sl.kind) {
          case UniformSlot::Double: o << "  const double " << slot_names[k] << " = " << P << "d[" << off << "];\n"; break;
          case UniformSlot::Float: o << "  const float " << eref(k) << " = " << P << "f[" << off << "];\n"; break;
          case UniformSlot::Bool: o << "  const bool " << eref(k) << " = " << P << "f[" << off << "] != 0.0f;\n"; break;
          case UniformSlot::DwPair:
            o << "  const mf_dw " << (ar == Ar::F32 ? slot_names[k] : eref(k)) << " = mf_dw_make(" << P << "f["
              << off << "], " << P << "f[" << sl.offset + 1 << "]);\n";
            break;
        }
      }
    };
    auto body = [&](std::ostringstream& o, const std::string& ind) {
      for (size_t i = 0; i < ns.size(); i++) {
        if (!live[i] || ns[i].uniform || ns[i].op == Op::Input) continue;
        const std::string st = estmt(int(i));
        if (!st.empty()) o << ind << st << "\n";
      }
    };
    // Accumulation of output j from the body's value (per thread).
    auto acc_decl = [&](std::ostringstream& o) {
      if (ar == Ar::F32 || ar == Ar::F32S)
        o << "  float acc[MF_NREG], cmp[MF_NREG];\n#pragma unroll\n  for (int j = 0; j < MF_NREG; j++) { acc[j] = 0.0f; cmp[j] = 0.0f; }\n";
      else if (ar == Ar::F64)
        o << "  double acc[MF_NREG];\n#pragma unroll\n  for (int j = 0; j < MF_NREG; j++) acc[j] = 0.0;\n";
      else
        o << "  mf_dw acc[MF_NREG];\n#pragma unroll\n  for (int j = 0; j < MF_NREG; j++) acc[j] = mf_dw_make(0.0f, 0.0f);\n";
      if (NREG < M) {  // this thread's column of the shared partials
        if (ar == Ar::F32 || ar == Ar::F32S)
          o << "  __shared__ float mf_sacc[MF_NOUT - MF_NREG][MF_BLOCK], mf_scmp[MF_NOUT - MF_NREG][MF_BLOCK];\n"
            << "  for (int j = 0; j < MF_NOUT - MF_NREG; j++) { mf_sacc[j][threadIdx.x] = 0.0f; "
               "mf_scmp[j][threadIdx.x] = 0.0f; }\n";
        else if (ar == Ar::F64)
          o << "  __shared__ double mf_sacc[MF_NOUT - MF_NREG][MF_BLOCK];\n"
            << "  for (int j = 0; j < MF_NOUT - MF_NREG; j++) mf_sacc[j][threadIdx.x] = 0.0;\n";
        else
          o << "  __shared__ mf_dw mf_sacc[MF_NOUT - MF_NREG][MF_BLOCK];\n"
            << "  for (int j = 0; j < MF_NOUT - MF_NREG; j++) mf_sacc[j][threadIdx.x] = mf_dw_make(0.0f, 0.0f);\n";
      }
      for (int j = 0; j < M; j++)
        if (logprod[j] >= 0) {
          o << "  mf_dw lpm" << j << " = mf_dw_make(1.0f, 0.0f);\n  int lpe" << j << " = 0;\n";
          if (logadd[j] >= 0) o << "  int lpc" << j << " = 0;\n";
        }
      if (has_addu) o << "  int mf_cnt = 0;  // events of this thread (for the x + u outputs)\n";
    };
    // A thread's partial of output j (and its FP32 compensation): a register
    // or the thread's slot of the shared partials.
    auto accref = [&](int j) {
      return j < NREG ? "acc[" + std::to_string(j) + "]"
                      : "mf_sacc[" + std::to_string(j - NREG) + "][threadIdx.x]";
    };
    auto cmpref = [&](int j) {
      return j < NREG ? "cmp[" + std::to_string(j) + "]"
                      : "mf_scmp[" + std::to_string(j - NREG) + "][threadIdx.x]";
    };
    // Per-thread partials of the log-product outputs, before the block reduction.
    auto acc_finish = [&](std::ostringstream& o) {
      for (int j = 0; j < M; j++)
        if (addu[j] >= 0)
          o << "  " << accref(j) << " = " << (addsign[j] > 0 ? "mf_dw_add" : "mf_dw_sub") << "(mf_dw_renorm("
            << accref(j) << "), mf_dw_mul(mf_dw_make((float)mf_cnt, 0.0f), " << eref(addu[j]) << "));\n";
      for (int j = 0; j < M; j++) {
        if (logprod[j] < 0) continue;
        const std::string J = std::to_string(j);
        o << "  { mf_dw q_ = mf_dw_logprod_log(lpm" << J << ", lpe" << J << ", mf_logtab);\n";
        if (logadd[j] >= 0) {
          // plus (minus) the thread's event count times u, the count exact in FP32
          std::string uw;
          if (ns[logadd[j]].op == Op::Const) {
            const float h = float(ns[logadd[j]].value);
            char b[96];
            std::snprintf(b, sizeof b, "mf_dw_make(%af, %af)", double(h),
                          double(float(ns[logadd[j]].value - double(h))));
            uw = b;
          } else {
            uw = ar == Ar::F32 ? "uw" + std::to_string(logadd[j]) : eref(logadd[j]);
          }
          o << "    const mf_dw c_ = mf_dw_mul(mf_dw_make((float)lpc" << J << ", 0.0f), " << uw << ");\n"
            << "    q_ = " << (logsign[j] > 0 ? "mf_dw_add" : "mf_dw_sub") << "(q_, c_);\n";
        }
        if (ar == Ar::F32)  // as a compensated FP32 partial: (acc, -cmp) = (h, l)
          o << "    " << accref(j) << " = q_.h; " << cmpref(j) << " = -q_.l; }\n";
        else
          o << "    " << accref(j) << " = q_; }\n";
      }
    };
    auto acc_one = [&](std::ostringstream& o, const std::string& ind, int j) {
      {
        if (logadd[j] >= 0) o << ind << "lpc" << j << "++;\n";
        if (ar == Ar::F32 && logprod[j] >= 0) {
          o << ind << "mf_dw_logprod(lpm" << j << ", lpe" << j << ", we" << logprod[j] << ");\n";
          return;
        }
        const std::string r = eref(accnode[j]);
        if (ar == Ar::F32 || ar == Ar::F32S)
          o << ind << "mf_kahan_f32(" << accref(j) << ", " << cmpref(j) << ", " << r << ");\n";
        else if (ar == Ar::F64)
          o << ind << accref(j) << " += " << r << ";\n";
        else if (logprod[j] >= 0)
          o << ind << "mf_dw_logprod(lpm" << j << ", lpe" << j << ", " << eref(logprod[j]) << ");\n";
        else if (fused[j].first >= 0)
          o << ind << "mf_dw_acc_mul(" << accref(j) << ", " << eref(fused[j].first) << ", "
            << eref(fused[j].second) << ");\n";
        else
          o << ind << "mf_dw_acc(" << accref(j) << ", " << r << ");\n";
      }
    };
    auto acc_add = [&](std::ostringstream& o, const std::string& ind) {
      for (int j = 0; j < M; j++) acc_one(o, ind, j);
    };
    // Kernels with many outputs (Hessians) accumulate each output as soon as
    // the values it needs exist, instead of after the whole body: the outputs'
    // values then need not all be live at once (105 for the S+P-wave Hessian,
    // two registers each in double-float). Same operations in the same order
    // per output, so the same sums.
    const bool interleave = M > 16;
    std::vector<std::vector<int>> ready_after(ns.size() + 1);  // [ns.size()]: before the first statement
    if (interleave) {
      auto in_body = [&](int id) { return id >= 0 && live[id] && !ns[id].uniform && ns[id].op != Op::Input; };
      for (int j = 0; j < M; j++) {
        std::vector<int> deps{accnode[j]};
        if (ar == Ar::F32 && logprod[j] >= 0)
          deps = {logprod[j]};
        else if (ar == Ar::DW && logprod[j] >= 0)
          deps = {logprod[j]};
        else if (ar == Ar::DW && fused[j].first >= 0)
          deps = {fused[j].first, fused[j].second};
        int at = -1;
        for (int d : deps)
          if (in_body(d)) at = std::max(at, d);
        ready_after[at < 0 ? ns.size() : size_t(at)].push_back(j);
      }
    }
    // The body and the accumulation of every output; `guard` (a condition, or
    // empty) decides whether this event counts.
    auto body_acc = [&](std::ostringstream& o, const std::string& ind, const std::string& guard) {
      if (has_addu) o << ind << (guard.empty() ? "" : "if (" + guard + ") ") << "mf_cnt++;\n";
      auto accs = [&](const std::vector<int>& js) {
        if (js.empty()) return;
        if (!guard.empty()) o << ind << "if (" << guard << ") {\n";
        for (int j : js) acc_one(o, guard.empty() ? ind : ind + "  ", j);
        if (!guard.empty()) o << ind << "}\n";
      };
      if (!interleave) {
        body(o, ind);
        std::vector<int> all(M);
        for (int j = 0; j < M; j++) all[j] = j;
        accs(all);
        return;
      }
      accs(ready_after[ns.size()]);
      for (size_t i = 0; i < ns.size(); i++) {
        if (!live[i] || ns[i].uniform || ns[i].op == Op::Input) continue;
        const std::string st = estmt(int(i));
        if (!st.empty()) o << ind << st << "\n";
        accs(ready_after[i]);
      }
    };
    // A thread's partial of output J as a double-float value (expression).
    auto thread_dw = [&](const std::string& J) -> std::string {
      auto one = [&](const std::string& a, const std::string& c) {
        if (ar == Ar::F32 || ar == Ar::F32S) return "mf_two_sum(" + a + ", -" + c + ")";
        if (ar == Ar::F64) return "mf_dw_split(" + a + ")";
        return "mf_dw_renorm(" + a + ")";
      };
      if (NREG == M) return one("acc[" + J + "]", "cmp[" + J + "]");
      // J is a constant once the loop is unrolled; both indices stay in bounds
      const std::string r = "((" + J + ") < MF_NREG ? (" + J + ") : 0)";
      const std::string sh = "[(" + J + ") < MF_NREG ? 0 : (" + J + ") - MF_NREG][threadIdx.x]";
      return "((" + J + ") < MF_NREG ? " + one("acc[" + r + "]", "cmp[" + r + "]") + " : " +
             one("mf_sacc" + sh, "mf_scmp" + sh) + ")";
    };
    // Block reduction of every output into mf_blk[] (shared): outputs go in
    // chunks of MF_RC through a [MF_RC][MF_BLOCK] staging array; warp w sums
    // output j0 + w (each lane a fixed stride of threads, then a shuffle
    // tree), so every output costs one warp's work instead of every warp's.
    // The order is fixed, so the result is reproducible.
    auto block_reduce = [&](std::ostringstream& o) {
      o << "  __shared__ float2 mf_stage_red[MF_RC][MF_BLOCK];\n  __shared__ float2 mf_blk[MF_NOUT];\n"
        << "  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;\n"
        << "#pragma unroll\n  for (int j0 = 0; j0 < MF_NOUT; j0 += MF_RC) {\n"
        << "#pragma unroll\n    for (int c = 0; c < MF_RC; c++)\n"
        << "      if (j0 + c < MF_NOUT) {\n        const mf_dw t = " << thread_dw("j0 + c") << ";\n"
        << "        mf_stage_red[c][threadIdx.x] = make_float2(t.h, t.l);\n      }\n"
        << "    __syncthreads();\n"
        << "    if (warp < MF_RC && j0 + warp < MF_NOUT) {\n"
        << "      mf_dw a = mf_dw_make(mf_stage_red[warp][lane].x, mf_stage_red[warp][lane].y);\n"
        << "#pragma unroll\n      for (int k = 1; k < MF_BLOCK / 32; k++)\n"
        << "        a = mf_dw_add(a, mf_dw_make(mf_stage_red[warp][lane + 32 * k].x, mf_stage_red[warp][lane + 32 * k].y));\n"
        << "#pragma unroll\n      for (int o = 16; o > 0; o >>= 1) a = mf_dw_add(a, mf_dw_shfl_xor(a, o));\n"
        << "      if (lane == 0) mf_blk[j0 + warp] = make_float2(a.h, a.l);\n    }\n"
        << "    __syncthreads();\n  }\n";
    };
    bool f32_logprod = false;
    for (int j = 0; j < M; j++) f32_logprod = f32_logprod || (ar == Ar::F32 && logprod[j] >= 0);
    auto load_table = [&](std::ostringstream& o) {
      if (f32_logprod) {
        o << "  __shared__ float4 mf_logtab[128];\n"
          << "  for (int q = threadIdx.x; q < 128; q += MF_BLOCK) mf_logtab[q] = mf_dw_logtab_g[q];\n"
          << "  __syncthreads();\n";
        return;
      }
      if (ar != Ar::DW || (!has_log && !has_exp)) return;
      if (has_log)
        o << "  __shared__ float4 mf_logtab[128];\n"
          << "  for (int q = threadIdx.x; q < 128; q += MF_BLOCK) mf_logtab[q] = mf_dw_logtab_g[q];\n";
      if (has_exp)
        o << "  __shared__ float2 mf_exptab[64];\n"
          << "  for (int q = threadIdx.x; q < 64; q += MF_BLOCK) mf_exptab[q] = mf_dw_exptab_g[q];\n";
      o << "  __syncthreads();\n";
    };
    auto input_value = [&](const std::string& raw) {
      if (ar == Ar::DW) return (pair ? "mf_dw_pair(" : "mf_dw_split(") + raw + ")";
      return raw;
    };
    const std::string DT = pair ? "float2" : ST;  // element type the REDUCE entries read
    const std::string XT = ar == Ar::F32 ? "float" : (ar == Ar::F64 || ar == Ar::F32S) ? "double" : "mf_dw";

    s << "struct mf_args { double d[" << out.nd << "]; float f[" << out.nf << "]; };\n";
    const auto entry_mark = s.tellp();
    // ---- single-dataset reduce ----
    s << "extern \"C\" __global__ void MF_BOUNDS " << out.entry << "(const " << DT
      << "* __restrict__ data, mf_u64 stride, mf_u64 n, mf_args P, float2* __restrict__ partials,"
      << " unsigned* __restrict__ counter, double* __restrict__ out, unsigned* __restrict__ status, unsigned seq) {\n";
    const auto body_mark = s.tellp();
    s << "  mf_launch_dependents();  // the next evaluation may start its event loop on SMs this grid frees\n";
    load_table(s);
    prologue(s, "P.");
    acc_decl(s);
    const std::string VT = V == 1 ? DT : pair ? "float4" : st32 ? (V == 4 ? "float4" : "float2") : "double2";
    const char* comp[4] = {"x", "y", "z", "w"};
    // event v of the vector loaded into l<k>
    auto lane_of = [&](int k, int v) -> std::string {
      const std::string l = "l" + std::to_string(k);
      if (pair) return V == 1 ? l : "make_float2(" + l + "." + comp[2 * v] + ", " + l + "." + comp[2 * v + 1] + ")";
      return V == 1 ? l : l + "." + comp[v];
    };
    auto emit_events = [&](const std::string& ind, const std::string& idx0, const std::string& valid_base,
                           const std::function<std::string(int)>& src) {
      for (int k : out.used_inputs) s << ind << "const " << VT << " l" << k << " = " << src(k) << ";\n";
      for (int v = 0; v < V; v++) {
        s << ind << "{\n";
        for (int k : out.used_inputs)
          s << ind << "  const " << XT << " x" << k << " = " << input_value(lane_of(k, v)) << ";\n";
        body_acc(s, ind + "  ", valid_base + " + " + std::to_string(v) + " < n");
        s << ind << "}\n";
      }
      (void)idx0;
    };
    const int NC = int(out.used_inputs.size());
    if (out.pipelined && NC > 0) {
      // Persistent blocks; tile t (events [t*MF_TILE, (t+1)*MF_TILE) of every
      // column read by the body) goes to block t % gridDim.x. Thread 0 keeps
      // MF_STAGES - 1 tiles in flight with bulk asynchronous copies into a
      // ring of shared-memory stages; all threads wait on the stage's
      // mbarrier (bounded), compute from shared memory and release the stage.
      const size_t es = st32 ? 4 : 8;  // float pairs are 8 bytes too
      out.smem_bytes = size_t(out.stages) * NC * out.tile * es;
      s << "#define MF_TILE " << out.tile << "\n#define MF_STAGES " << out.stages << "\n#define MF_NC " << NC << "\n";
      s << "  extern __shared__ __align__(128) unsigned char mf_dyn[];\n";
      s << "  " << DT << "* __restrict__ stage = reinterpret_cast<" << DT << "*>(mf_dyn);\n";
      s << "  __shared__ __align__(8) unsigned long long mf_bar[MF_STAGES];\n";
      s << "  const mf_u64 ntiles = (n + MF_TILE - 1) / MF_TILE;\n";
      s << "  if (threadIdx.x == 0) {\n    for (int q = 0; q < MF_STAGES; q++) mf_mbar_init(&mf_bar[q], 1u);\n"
        << "    mf_fence_mbar_init();\n  }\n  __syncthreads();\n";
      // issue lambda as a macro-like block
      std::ostringstream issue;
      issue << "{ const mf_u64 t0 = (TL) * (mf_u64)MF_TILE; mf_u64 cnt = stride - t0; if (cnt > MF_TILE) cnt = MF_TILE;\n"
            << "          const unsigned bytes = (unsigned)(cnt * sizeof(" << DT << "));\n"
            << "          mf_mbar_expect_tx(&mf_bar[SL], bytes * MF_NC);\n";
      for (int ci = 0; ci < NC; ci++)
        issue << "          mf_bulk_g2s(stage + ((mf_u64)(SL) * MF_NC + " << ci << ") * MF_TILE, data + (mf_u64)"
              << out.used_inputs[ci] << " * stride + t0, bytes, &mf_bar[SL]);\n";
      issue << "        }";
      auto issue_code = [&](const std::string& tl, const std::string& sl) {
        std::string c = issue.str();
        for (size_t p; (p = c.find("(TL)")) != std::string::npos;) c.replace(p, 4, "(" + tl + ")");
        for (size_t p; (p = c.find("SL")) != std::string::npos;) c.replace(p, 2, sl);
        return c;
      };
      s << "  unsigned issued = 0;  // tiles issued by thread 0 (valid in thread 0)\n";
      s << "  if (threadIdx.x == 0)\n    for (int q = 0; q < MF_STAGES - 1; q++) {\n"
        << "      const mf_u64 tl = blockIdx.x + (mf_u64)q * gridDim.x;\n      if (tl < ntiles) {\n        "
        << issue_code("tl", "q") << "\n        issued++;\n      }\n    }\n";
      s << "  unsigned it = 0;\n  bool aborted = false;\n";
      s << "  for (mf_u64 tile = blockIdx.x; tile < ntiles; tile += gridDim.x, it++) {\n";
      s << "    const unsigned sl = it % MF_STAGES, par = (it / MF_STAGES) & 1u;\n";
      s << "    if (threadIdx.x == 0) {\n      const mf_u64 nt = tile + (mf_u64)(MF_STAGES - 1) * gridDim.x;\n"
        << "      if (nt < ntiles) {\n        const unsigned ns = (it + MF_STAGES - 1) % MF_STAGES;\n"
        << "        mf_fence_proxy_async();\n        " << issue_code("nt", "ns") << "\n        issued++;\n      }\n    }\n";
      s << "    const bool ok = mf_mbar_wait_bounded(&mf_bar[sl], par);\n";
      s << "    if (__syncthreads_or(!ok)) { aborted = true; break; }\n";
      s << "    const " << DT << "* __restrict__ sb = stage + (mf_u64)sl * MF_NC * MF_TILE;\n";
      s << "    const mf_u64 tbase = tile * (mf_u64)MF_TILE;\n";
      s << "    {\n      const int e0 = threadIdx.x * " << V << ";\n";
      std::map<int, int> colpos;
      for (int ci = 0; ci < NC; ci++) colpos[out.used_inputs[ci]] = ci;
      emit_events("      ", "e0", "tbase + e0", [&](int k) {
        return "*reinterpret_cast<const " + VT + "*>(sb + " + std::to_string(colpos[k]) + " * MF_TILE + e0)";
      });
      s << "    }\n    __syncthreads();\n  }\n";
      // abort: report, drain this block's copies still in flight (bounded), continue to the reduction
      s << "  if (aborted && threadIdx.x == 0) {\n    atomicOr(status, 1u);\n"
        << "    for (unsigned k = it; k < issued; k++) mf_mbar_wait_bounded(&mf_bar[k % MF_STAGES], (k / MF_STAGES) & 1u);\n"
        << "  }\n";
    } else {
      s << "  const mf_u64 step = (mf_u64)gridDim.x * MF_BLOCK * " << V << ";\n";
      // unrolled: the next iteration's loads are issued before this one's arithmetic
      if (out.stages > 1) s << "#pragma unroll " << out.stages << "\n";
      s << "  for (mf_u64 base = ((mf_u64)blockIdx.x * MF_BLOCK + threadIdx.x) * " << V
        << "; base < n; base += step) {\n";
      emit_events("    ", "base", "base", [&](int k) {
        return "__ldg(reinterpret_cast<const " + VT + "*>(data + (mf_u64)" + std::to_string(k) + " * stride + base))";
      });
      s << "  }\n";
    }
    s << "  __shared__ float2 red[MF_NOUT][MF_BLOCK / 32];\n  __shared__ bool am_last;\n";
    acc_finish(s);
    block_reduce(s);
    // the per-block work, shared by the single-evaluation and the batched entry
    const std::string body_text = s.str().substr(size_t(body_mark));
    // Fixed-order double-float combine of mf_nb partial rows (partials) into
    // out[]: thread t takes rows t, t + MF_BLOCK, ... for every output (all
    // loads of a round issued before the adds), then a warp tree and a pass
    // over the warps in order. The order depends only on mf_nb, the grid size
    // of the evaluation. Uses red[][], lane and warp.
    // Outputs are combined MF_CC at a time (registers O(MF_CC), not
    // O(MF_NOUT)); within each output the order is the one above, so the
    // chunking changes no result.
    const std::string combine_text = R"CUDA(  {
    for (int j0 = 0; j0 < MF_NOUT; j0 += MF_CC) {
      mf_dw s[MF_CC];
#pragma unroll
      for (int c = 0; c < MF_CC; c++) s[c] = mf_dw_make(0.0f, 0.0f);
      for (unsigned b0 = 0; b0 < mf_nb; b0 += MF_Q * MF_BLOCK) {
        float2 v[MF_Q][MF_CC];
#pragma unroll
        for (int q = 0; q < MF_Q; q++) {
          const unsigned b = b0 + q * MF_BLOCK + threadIdx.x;
#pragma unroll
          for (int c = 0; c < MF_CC; c++)
            v[q][c] = (b < mf_nb && j0 + c < MF_NOUT) ? __ldcg(partials + (mf_u64)b * MF_NOUT + j0 + c)
                                                        : make_float2(0.0f, 0.0f);
        }
#pragma unroll
        for (int q = 0; q < MF_Q; q++)
#pragma unroll
          for (int c = 0; c < MF_CC; c++) s[c] = mf_dw_add(s[c], mf_dw_make(v[q][c].x, v[q][c].y));
      }
#pragma unroll
      for (int c = 0; c < MF_CC; c++) {
        if (j0 + c >= MF_NOUT) break;
        mf_dw a = s[c];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) a = mf_dw_add(a, mf_dw_shfl_xor(a, o));
        if (lane == 0) red[j0 + c][warp] = make_float2(a.h, a.l);
      }
    }
    __syncthreads();
    for (int j = threadIdx.x; j < MF_NOUT; j += MF_BLOCK) {
      mf_dw b = mf_dw_make(red[j][0].x, red[j][0].y);
      for (int w = 1; w < MF_BLOCK / 32; w++) b = mf_dw_add(b, mf_dw_make(red[j][w].x, red[j][w].y));
      out[j] = mf_dw_to_double(b);
    }
  }
)CUDA";
    s << R"CUDA(  // Launched as a programmatic dependent of the previous evaluation on the
  // stream (batched evaluations), this grid ran its event loop while that
  // one finished; the scratch below is shared, so wait for it to complete.
  mf_grid_dependency_wait();
  for (int j = threadIdx.x; j < MF_NOUT; j += MF_BLOCK) partials[(mf_u64)blockIdx.x * MF_NOUT + j] = mf_blk[j];
  // Completion count with release/acquire semantics: the barrier orders the
  // block's partial writes before thread 0's release; the last block's
  // acquire plus the barrier orders its reads of every partial after.
  __syncthreads();
  if (threadIdx.x == 0) am_last = (mf_atom_add_acq_rel(counter, 1u) == gridDim.x - 1);
  __syncthreads();
  if (!am_last) return;
  const unsigned mf_nb = gridDim.x;
)CUDA" << combine_text << R"CUDA(  if (threadIdx.x == 0) *counter = 0u;
  // Synchronous evaluation (seq != 0): out[] is mapped host memory; publish
  // completion in the mapped word status[1] after every output is visible
  // system-wide, so the host can read the sums without a stream synchronize.
  if (seq != 0u) {
    __threadfence_system();
    __syncthreads();
    if (threadIdx.x == 0) *reinterpret_cast<volatile unsigned*>(status + 1) = seq;
  }
)CUDA";
    if (!out.pipelined) {
      std::string work = s.str().substr(size_t(body_mark));
      auto replace_all = [](std::string& t, const std::string& from, const std::string& to) {
        for (size_t p = t.find(from); p != std::string::npos; p = t.find(from, p + to.size())) t.replace(p, from.size(), to);
      };
      replace_all(work, "blockIdx.x", "mf_vb");
      replace_all(work, "gridDim.x", "mf_grid");
      out.resident_prefix = s.str().substr(0, size_t(entry_mark));
      out.resident_data_type = DT;
      out.resident_body = "__device__ __forceinline__ void mf_rbody(const " + DT +
                          "* __restrict__ data, mf_u64 stride, mf_u64 n, const mf_args& P, float2* __restrict__ "
                          "partials, unsigned* __restrict__ counter, double* __restrict__ out, unsigned* "
                          "__restrict__ status, unsigned seq, unsigned mf_vb, unsigned mf_grid) {\n" +
                          work + "}\n";
    }
    s << "}\n";
    // ---- batched evaluations: per-block partials only, then one combine ----
    // Evaluation e of a batch writes its partial rows to its own slot of the
    // batch's partial buffer without counting or combining, so consecutive
    // evaluations' grids overlap (each waits for its predecessor only after
    // its own work); <entry>_combine then reduces every evaluation's rows
    // (one block each, the same fixed order: the sums equal the
    // single-evaluation entry's).
    s << "extern \"C\" __global__ void MF_BOUNDS " << out.entry << "_part(const " << DT
      << "* __restrict__ data, mf_u64 stride, mf_u64 n, mf_args P, float2* __restrict__ partials,"
      << " unsigned* __restrict__ status) {\n"
      << body_text
      << "  for (int j = threadIdx.x; j < MF_NOUT; j += MF_BLOCK) partials[(mf_u64)blockIdx.x * MF_NOUT + j] = mf_blk[j];\n"
      << "  // complete only after the previous evaluation's grid: completions stay in\n"
      << "  // stream order, so the combine launch after the last evaluation sees every partial\n"
      << "  mf_grid_dependency_wait();\n"
      << "}\n";
    s << "extern \"C\" __global__ void __launch_bounds__(MF_BLOCK) " << out.entry
      << "_combine(const float2* __restrict__ partials_all, mf_u64 pstride, const unsigned* __restrict__ grids,"
      << " double* __restrict__ out_all, unsigned count, unsigned grid_all) {\n"
      << "  // launched as a programmatic dependent of the last evaluation: its partials\n"
      << "  // (and every earlier one's) are complete and visible after this\n"
      << "  mf_grid_dependency_wait();\n"
      << "  const unsigned e = blockIdx.x;\n  if (e >= count) return;\n"
      << "  // every evaluation's grid size, or (grids null) the one they all share\n"
      << "  const unsigned mf_nb = grids ? grids[e] : grid_all;\n"
      << "  const float2* __restrict__ partials = partials_all + (mf_u64)e * pstride;\n"
      << "  double* __restrict__ out = out_all + (mf_u64)e * MF_NOUT;\n"
      << "  __shared__ float2 red[MF_NOUT][MF_BLOCK / 32];\n"
      << "  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;\n"
      << combine_text << "}\n";

    // ---- ragged segments: one block per segment ----
    s << "extern \"C\" __global__ void __launch_bounds__(MF_BLOCK) " << out.entry << "_segments(const " << DT
      << "* __restrict__ data, mf_u64 stride, const mf_u64* __restrict__ seg_begin,"
      << " const unsigned* __restrict__ seg_count, const mf_args* __restrict__ args,"
      << " double* __restrict__ out) {\n";
    load_table(s);
    s << "  const unsigned seg = blockIdx.x;\n  const mf_u64 first = seg_begin[seg];\n"
      << "  const mf_u64 cnt = seg_count[seg];\n  const mf_args& P = args[seg];\n";
    prologue(s, "P.");
    acc_decl(s);
    s << "  for (mf_u64 i = threadIdx.x; i < cnt; i += MF_BLOCK) {\n";
    for (int k : out.used_inputs)
      s << "    const " << XT << " x" << k << " = " << input_value("__ldg(data + (mf_u64)" + std::to_string(k) +
                                                                   " * stride + first + i)")
        << ";\n";
    body_acc(s, "    ", "");
    s << "  }\n";
    acc_finish(s);
    block_reduce(s);
    s << R"CUDA(  for (int j = threadIdx.x; j < MF_NOUT; j += MF_BLOCK)
    out[(mf_u64)seg * MF_NOUT + j] = mf_dw_to_double(mf_dw_make(mf_blk[j].x, mf_blk[j].y));
}
)CUDA";
    // ---- many datasets in one launch: one block per segment ----
    // A segment is a run of at most MF_MULTI_CHUNK events of one dataset
    // (its own columns, stride and parameter row); the block writes its
    // partial row to `row` of the partial buffer, and <entry>_combine then
    // reduces each dataset's rows in a fixed order. A dataset's sums depend
    // only on its own events, parameters and size (segments are cut at fixed
    // multiples of MF_MULTI_CHUNK), never on what else shares the launch.
    s << "struct mf_seg { const void* data; mf_u64 stride; mf_u64 first; unsigned count; unsigned req; unsigned row;"
         " unsigned pad; };\n";
    s << "extern \"C\" __global__ void __launch_bounds__(MF_BLOCK) " << out.entry
      << "_multi(const mf_seg* __restrict__ segs, const mf_args* __restrict__ args,"
      << " float2* __restrict__ partials) {\n";
    load_table(s);
    s << "  const mf_seg S = segs[blockIdx.x];\n"
      << "  const " << DT << "* __restrict__ data = static_cast<const " << DT << "*>(S.data);\n"
      << "  const mf_u64 stride = S.stride, first = S.first;\n  const unsigned cnt = S.count;\n"
      << "  const mf_args& P = args[S.req];\n";
    prologue(s, "P.");
    acc_decl(s);
    s << "  for (unsigned i = threadIdx.x; i < cnt; i += MF_BLOCK) {\n";
    for (int k : out.used_inputs)
      s << "    const " << XT << " x" << k << " = " << input_value("__ldg(data + (mf_u64)" + std::to_string(k) +
                                                                   " * stride + first + i)")
        << ";\n";
    body_acc(s, "    ", "");
    s << "  }\n";
    acc_finish(s);
    block_reduce(s);
    s << R"CUDA(  for (int j = threadIdx.x; j < MF_NOUT; j += MF_BLOCK) partials[(mf_u64)S.row * MF_NOUT + j] = mf_blk[j];
}
)CUDA";
    // ---- per-dataset preparation of the columns the entries above read ----
    if (prep) {
      const std::string PT = pair ? "float2" : ST;
      s << "extern \"C\" __global__ void __launch_bounds__(256) " << out.entry << "_prep(const " << ST
        << "* __restrict__ data, mf_u64 stride, mf_u64 n, " << PT << "* __restrict__ outp) {\n"
        << "  for (mf_u64 i = (mf_u64)blockIdx.x * 256 + threadIdx.x; i < stride; i += (mf_u64)gridDim.x * 256) {\n"
        << "    const bool v = i < n;  // padding events are written as zeros\n";
      auto src = [&](int col) {
        return "(double)__ldg(data + (mf_u64)" + std::to_string(col) + " * stride + i)";
      };
      for (size_t m = 0; m < fold.cols.size(); m++) {
        const auto& terms = fold.cols[m];
        s << "    {\n      double y = 0.0;\n      if (v) {\n        y = " << src(terms[0].first) << ";\n";
        for (size_t t = 1; t < terms.size(); t++) {
          const double c = terms[t].second;
          if (c == 1.0)
            s << "        y = __dadd_rn(y, " << src(terms[t].first) << ");\n";
          else if (c == -1.0)
            s << "        y = __dsub_rn(y, " << src(terms[t].first) << ");\n";
          else
            s << "        y = __fma_rn(" << fmt_const(c, false) << ", " << src(terms[t].first) << ", y);\n";
        }
        s << "      }\n";
        if (pair)
          s << "      const mf_dw w = mf_dw_split(y);\n      outp[(mf_u64)" << m << " * stride + i] = make_float2(w.h, w.l);\n";
        else
          s << "      outp[(mf_u64)" << m << " * stride + i] = (" << PT << ")y;\n";
        s << "    }\n";
      }
      s << "  }\n}\n";
    }
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
    if (!ar32) s << dw_log_table() << kDwPrelude;
    s << "extern \"C\" __global__ void __launch_bounds__(MF_BLOCK) " << out.entry
      << "(const unsigned* __restrict__ seeds, unsigned nseeds, mf_u64 n, mf_u64 nper, mf_par P, " << ST
      << "* __restrict__ outp, mf_u64 out_stride, unsigned* __restrict__ status, unsigned long long max_tries,"
      << " unsigned long long splitmix_seed) {\n";
    s << "  const unsigned t = blockIdx.x * MF_BLOCK + threadIdx.x;\n  if (t >= nseeds) return;\n";
    // the stream's xoshiro128++ state: from the seed table, or (seeds null)
    // made here as mf_splitmix_seed_rows makes row t: the upper halves of four
    // SplitMix64 outputs (Steele, Lea and Flood, OOPSLA 2014) from
    // (seed mod 2^32) * 2^32 + t
    s << "  unsigned st[4];\n"
      << "  if (seeds) {\n#pragma unroll\n    for (int k = 0; k < 4; k++) st[k] = seeds[(mf_u64)k * nseeds + t];\n"
      << "  } else {\n    unsigned long long sm = (splitmix_seed & 0xffffffffull) * 4294967296ull + t;\n"
      << "#pragma unroll\n    for (int k = 0; k < 4; k++) {\n"
      << "      unsigned long long z = (sm += 0x9e3779b97f4a7c15ull);\n"
      << "      z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;\n"
      << "      z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;\n"
      << "      st[k] = (unsigned)((z ^ (z >> 31)) >> 32);\n    }\n  }\n";
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
    // FP64 generation: the density is evaluated in double-float (FP32
    // pairs on the FP32 pipe, which GB300 issues at 64x its FP64 rate:
    // proposals split with integer operations, parameter-only values
    // converted once per thread, tables from global memory), and the accept
    // decision maxprob*u < p is recomputed with the density in exact FP64
    // (the code the reference runs) whenever |maxprob*u - p| is within
    // 1e-9 * maxprob or p is not finite. The double-float density is within
    // about 1e-13 of the exact one when its intermediates stay inside the
    // FP32 exponent range (2^-100 to 3.4e38 in magnitude, or zero), far
    // inside that margin, so every decision -- and every generated event --
    // equals the FP64 one. Only the proposals, the bound and the comparison
    // stay on the FP64 pipe.
    const bool fast_density = !ar32;
    auto wref = [&](int id) -> std::string {
      const Node& n = ns[id];
      if (n.op == Op::Const) {
        const float h = float(n.value);
        const float l = float(n.value - double(h));
        char b[96];
        std::snprintf(b, sizeof b, "mf_dw_make(%af, %af)", double(h), double(l));
        return b;
      }
      if (n.op == Op::Input) return "xw" + std::to_string(n.index);
      if (n.op == Op::Param) return "pw" + std::to_string(n.index);
      if (n.uniform) return "uw" + std::to_string(id);
      return "w" + std::to_string(id);
    };
    // sin and cos of one operand share a reduction: operand -> (sin node, cos node)
    std::map<int, std::pair<int, int>> wsincos;
    {
      std::map<int, int> sin_of, cos_of;
      for (size_t i = 0; i < ns.size(); i++) {
        if (!live[i] || ns[i].uniform) continue;
        if (ns[i].op == Op::Sin) sin_of[ns[i].a] = int(i);
        if (ns[i].op == Op::Cos) cos_of[ns[i].a] = int(i);
      }
      for (auto& [a, si] : sin_of) {
        auto c = cos_of.find(a);
        if (c != cos_of.end()) wsincos[a] = {si, c->second};
      }
    }
    auto wstmt = [&](int id) -> std::string {
      const Node& n = ns[id];
      const std::string lhs = "const " + std::string(n.op == Op::Cmp ? "bool" : "mf_dw") + " w" + std::to_string(id) + " = ";
      const std::string A = n.a >= 0 ? wref(n.a) : "", B = n.b >= 0 ? wref(n.b) : "", Cc = n.c >= 0 ? wref(n.c) : "";
      auto D = [](const std::string& v) { return "mf_dw_to_double(" + v + ")"; };
      switch (n.op) {
        case Op::Add: return lhs + "mf_dw_add(" + A + ", " + B + ");";
        case Op::Sub: return lhs + "mf_dw_sub(" + A + ", " + B + ");";
        case Op::Mul: return lhs + "mf_dw_mul(" + A + ", " + B + ");";
        case Op::Div: return lhs + "mf_dw_mul(" + A + ", mf_dw_rcp(" + B + "));";
        case Op::Neg: return lhs + "mf_dw_neg(" + A + ");";
        case Op::Rcp: return lhs + "mf_dw_rcp(" + A + ");";
        case Op::Log: return lhs + "mf_dw_log(" + A + ", mf_dw_logtab_g);";
        case Op::Exp: return lhs + "mf_dw_exp(" + A + ", mf_dw_exptab_g);";
        case Op::Pow: return lhs + "mf_dw_pow(" + A + ", " + B + ", mf_dw_logtab_g, mf_dw_exptab_g);";
        case Op::Sqrt: return lhs + "mf_dw_sqrt(" + A + ");";
        case Op::Sin:
        case Op::Cos: {
          auto it = wsincos.find(n.a);
          if (it == wsincos.end()) return lhs + (n.op == Op::Sin ? "mf_dw_sin(" : "mf_dw_cos(") + A + ");";
          if (id != std::min(it->second.first, it->second.second)) return "";  // defined with the first of the two
          const std::string sn = "w" + std::to_string(it->second.first), cn = "w" + std::to_string(it->second.second);
          return "mf_dw " + sn + ", " + cn + "; mf_dw_sincos(" + A + ", &" + sn + ", &" + cn + ");";
        }
        case Op::Cmp:
          switch (n.cmp) {
            case CmpOp::Gt: return lhs + "mf_dw_gt(" + A + ", " + B + ");";
            case CmpOp::Lt: return lhs + "mf_dw_lt(" + A + ", " + B + ");";
            case CmpOp::Ge: return lhs + "mf_dw_ge(" + A + ", " + B + ");";
            case CmpOp::Le: return lhs + "mf_dw_le(" + A + ", " + B + ");";
            case CmpOp::Eq: return lhs + "mf_dw_eq(" + A + ", " + B + ");";
            case CmpOp::Ne: return lhs + "!mf_dw_eq(" + A + ", " + B + ");";
          }
          break;
        case Op::Select: return lhs + "(" + A + " ? " + B + " : " + Cc + ");";
        default:
          if (is_unary_fn(n.op)) return lhs + "mf_dw_from_double(" + fn_name(n.op, false) + "(" + D(A) + "));";
      }
      throw std::runtime_error("emit: unexpected node");
    };
    // parameter-only values the double-float density reads, converted once per thread
    auto emit_uniform_pairs = [&]() {
      std::set<int> uni;
      auto note = [&](int k) {
        if (k >= 0 && ns[k].uniform && ns[k].op != Op::Const) uni.insert(k);
      };
      for (size_t i = 0; i < ns.size(); i++) {
        if (!live[i] || ns[i].uniform || ns[i].op == Op::Input) continue;
        note(ns[i].a);
        note(ns[i].b);
        note(ns[i].c);
      }
      for (int r : roots) note(r);
      for (int k : uni) s << "  const mf_dw " << wref(k) << " = mf_dw_from_double(" << em.ref(k, "u") << ");\n";
    };
    auto accept_reject = [&]() {
      if (fast_density) emit_uniform_pairs();
      s << "  unsigned long long tries = 0;\n";
      s << "  for (mf_u64 i = from; i < to; i++) {\n    for (;;) {\n";
      s << "      if (++tries > max_tries) { atomicOr(status, 1u); return; }\n";
      for (int d = 0; d < D; d++) {
        s << "      const " << AT << " x" << d << " = " << add << "(" << fmt_const(printed15(gen->lo[d]), ar32) << ", "
          << mul << "(" << fmt_const(printed15(gen->hi[d] - gen->lo[d]), ar32) << ", (" << AT
          << ")(mf_xoshiro(st) * 2.3283064365386963e-10)));\n";
      }
      if (fast_density) {
        for (int d = 0; d < D; d++) s << "      const mf_dw xw" << d << " = mf_dw_split_rn(x" << d << ");\n";
        for (size_t i = 0; i < ns.size(); i++) {
          if (!live[i] || ns[i].uniform || ns[i].op == Op::Input) continue;
          const std::string st = wstmt(int(i));
          if (!st.empty()) s << "      " << st << "\n";
        }
        s << "      const double mf_ug = " << mul << "(maxprob, (double)(mf_xoshiro(st) * 2.3283064365386963e-10));\n";
        s << "      double mf_p = mf_dw_to_double_bits(" << wref(roots[0]) << ");\n";
        s << "      if (!(fabs(mf_ug - mf_p) > 1e-9 * maxprob) || isinf(mf_p)) {  // exact FP64 density\n";
        emit_body(s, "        ");
        s << "        mf_p = r0;\n      }\n";
        s << "      if (mf_ug < mf_p) {\n";
      } else {
        emit_body(s, "      ");
        s << "      if (" << mul << "(maxprob, (" << AT << ")(mf_xoshiro(st) * 2.3283064365386963e-10)) < r0) {\n";
      }
      for (int d = 0; d < D; d++)
        s << "        outp[(mf_u64)" << d << " * out_stride + i] = (" << ST << ")x" << d << ";\n";
      s << "        break;\n      }\n    }\n  }\n}\n";
    };
    s << "  const " << AT << " maxprob = " << fmt_const(printed15(gen->maxprob), ar32) << ";\n";
    s << "  const mf_u64 from = (mf_u64)t * nper;\n  mf_u64 to = from + nper; if (to > n) to = n;\n";
    accept_reject();
    // Segments (toy studies): `threads_per_seg` streams per segment; segment
    // s owns events [seg_begin[s], seg_begin[s] + seg_count[s]) and generates
    // them with its own parameter row and bound (thread r of the segment
    // takes the r-th block of ceil(count / threads_per_seg) events).
    s << "extern \"C\" __global__ void __launch_bounds__(MF_BLOCK) " << out.entry
      << "_segments(const unsigned* __restrict__ seeds, unsigned nthreads, unsigned threads_per_seg,"
      << " const mf_u64* __restrict__ seg_begin, const unsigned* __restrict__ seg_count,"
      << " const mf_par* __restrict__ seg_params, const double* __restrict__ seg_maxprob, " << ST
      << "* __restrict__ outp, mf_u64 out_stride, unsigned* __restrict__ status, unsigned long long max_tries) {\n";
    s << "  const unsigned t = blockIdx.x * MF_BLOCK + threadIdx.x;\n  if (t >= nthreads) return;\n";
    s << "  const unsigned seg = t / threads_per_seg, r = t - seg * threads_per_seg;\n";
    s << "  unsigned st[4];\n#pragma unroll\n  for (int k = 0; k < 4; k++) st[k] = seeds[(mf_u64)k * nthreads + t];\n";
    s << "  const mf_par& P = seg_params[seg];\n";
    emit_params_and_uniform(s, "P.v");
    s << "  const " << AT << " maxprob = (" << AT << ")seg_maxprob[seg];\n";
    s << "  const mf_u64 cnt = seg_count[seg], per = (cnt + threads_per_seg - 1) / threads_per_seg;\n";
    s << "  const mf_u64 from = seg_begin[seg] + (mf_u64)r * per;\n";
    s << "  mf_u64 to = from + per; if (to > seg_begin[seg] + cnt) to = seg_begin[seg] + cnt;\n";
    accept_reject();
  }
  out.source = s.str();
  return out;
}


void LoweredKernel::fill_args(const double* params, size_t np, unsigned char* out) const {
  fill_args_many(params, np, 1, out);
}

void LoweredKernel::fill_args_many(const double* params, size_t np, size_t count, unsigned char* out) const {
  // Straight-line evaluation of the nodes the slots read (both arms of a
  // select are evaluated; their values only feed the select), into a scratch
  // array of which only those entries are written and read; one scratch for
  // all rows.
  std::vector<double> val(nodes.size());
  const size_t ab = args_bytes();
  for (size_t r = 0; r < count; r++) {
    const double* pr = params + r * np;
    unsigned char* o = out + r * ab;
    std::memset(o, 0, ab);
    for (int id : eval_order) {
      const Node& n = nodes[id];
      double v;
      switch (n.op) {
        case Op::Const: v = n.value; break;
        case Op::Param: v = size_t(n.index) < np ? pr[n.index] : 0.0; break;
        case Op::Input: throw std::runtime_error("input column in a parameter-only value");
        case Op::Add: v = val[n.a] + val[n.b]; break;
        case Op::Sub: v = val[n.a] - val[n.b]; break;
        case Op::Mul: v = val[n.a] * val[n.b]; break;
        case Op::Div: case Op::Pow: v = apply_binary(n.op, val[n.a], val[n.b]); break;
        case Op::Cmp: v = apply_cmp(n.cmp, val[n.a], val[n.b]) ? 1.0 : 0.0; break;
        case Op::Select: v = val[n.a] != 0.0 ? val[n.b] : val[n.c]; break;
        default: v = apply_unary(n.op, val[n.a]); break;
      }
      val[id] = v;
    }
    double* d = reinterpret_cast<double*>(o);
    float* f = reinterpret_cast<float*>(o + size_t(nd) * 8);
    for (const auto& sl : slots) {
      const double v = val[sl.node];
      switch (sl.kind) {
        case UniformSlot::Double: d[sl.offset] = v; break;
        case UniformSlot::Float: f[sl.offset] = float(v); break;
        case UniformSlot::Bool: f[sl.offset] = v != 0.0 ? 1.0f : 0.0f; break;
        case UniformSlot::DwPair: {
          const float h = float(v);
          f[sl.offset] = h;
          f[sl.offset + 1] = float(v - double(h));
          break;
        }
      }
    }
  }
}

}  // namespace mf
