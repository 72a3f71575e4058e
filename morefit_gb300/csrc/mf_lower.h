// Lowering of MoreFit kernel expressions to CUDA C.
//
// Input: the C-syntax strings that ComputeGraphNode::get_kernel() prints
// (reference include/graph.hh: Sum "(a+b)" :314-320, Prod "(a*b)" :548-554,
// Exp/Log/Sqrt/Sin/... "f(x)" :786,987,1350,1451, Inv "1.0/(x)" :886, Neg
// "-(x)" :1253, Pow "pow(a,b)" :1094-1099, Conditional "((x==0.0) ? a : b)"
// :2270-2290, Constant "%.15e" :245-254, Variable name :2172).
//
// The strings of all outputs of one kernel are parsed into one hash-consed
// DAG, so a subexpression that several outputs share (the density p, its
// reciprocal, exp(...) terms) is evaluated once per event. Divisions become
// multiplications by a shared reciprocal. Nodes that depend only on
// parameters and constants are evaluated once per thread before the event
// loop. Only the input columns the expressions reference are loaded.
#ifndef MF_LOWER_H
#define MF_LOWER_H

#include <cstdint>
#include <map>
#include <memory>
#include <string>
#include <vector>

namespace mf {

enum class Op : uint8_t {
  Const, Input, Param, Add, Sub, Mul, Neg, Rcp, Div, Exp, Log, Sqrt, Sin, Cos, Tan, Asin, Acos, Atan, Erf,
  Pow, Cmp, Select
};
enum class CmpOp : uint8_t { Eq, Ne, Gt, Lt, Ge, Le };

struct Node {
  Op op;
  CmpOp cmp = CmpOp::Eq;
  double value = 0.0;  // Const
  int index = -1;      // Input column / Param slot
  int a = -1, b = -1, c = -1;
  bool uniform = true;  // depends on no input column
};

class Dag {
 public:
  Dag(const std::vector<std::string>& inputs, const std::vector<std::string>& params);
  // Parses one expression; returns the root node id. Throws std::runtime_error.
  int parse(const std::string& expr);
  const std::vector<Node>& nodes() const { return nodes_; }
  int input_count() const { return int(inputs_.size()); }
  const std::vector<std::string>& input_names() const { return inputs_; }
  const std::vector<std::string>& param_names() const { return params_; }
  // Node constructors with local simplification and hash-consing.
  int constant(double v);
  int unary(Op op, int a);
  int binary(Op op, int a, int b);
  int compare(CmpOp cmp, int a, int b);
  int select(int cond, int a, int b);
  // Host evaluation (parameter-only expressions, tests).
  double eval(int id, const std::vector<double>& inputs, const std::vector<double>& params) const;
  // Every node in order (children before parents) for one parameter vector;
  // inputs evaluate to 0. `vals` is resized to the node count.
  void eval_all(const double* params, size_t np, std::vector<double>& vals) const;

 private:
  int intern(const Node& n);
  std::vector<Node> nodes_;
  std::map<std::string, int> table_;
  std::vector<std::string> inputs_, params_;
  std::map<std::string, int> input_idx_, param_idx_;
};

// A parameter-only value the REDUCE body needs, evaluated on the host at
// launch and passed in the kernel's argument struct
// { double d[nd]; float f[nf]; }.
struct UniformSlot {
  enum Kind { Double = 0, Float = 1, DwPair = 2, Bool = 3 };
  int node;    // DAG node (a Param or a uniform node)
  int kind;
  int offset;  // index into d[] (Double) or f[] (others)
};

struct LoweredKernel {
  std::string source;            // complete CUDA C translation unit
  std::string entry;             // __global__ function name
  std::vector<int> used_inputs;  // input columns read by the kernel
  int vec = 1;                   // events per thread per iteration
  int block = 256;
  int acc_reg = 0;               // REDUCE: outputs whose per-thread partials are registers (the rest: shared memory)
  // REDUCE kernels stream tiles of `tile` events through `stages` shared-memory
  // buffers with bulk asynchronous copies (pipelined = true) or read global
  // memory directly (pipelined = false).
  bool pipelined = false;
  int tile = 0, stages = 0;
  // REDUCE kernels with direct loads: the single-evaluation entry's work as a
  // device function for a resident module (mf_runtime.cpp), which holds one
  // grid on the device and runs evaluations posted by the host:
  // resident_prefix is the translation unit up to the entry points (helpers,
  // macros, the argument struct), resident_body defines
  //   mf_rbody(data, stride, n, const mf_args& P, partials, counter, out,
  //            status, seq, unsigned block, unsigned grid)
  // doing block `block` of a grid of `grid` blocks, i.e. the entry with
  // blockIdx.x and gridDim.x replaced. Empty when not available.
  std::string resident_prefix, resident_body;
  std::string resident_data_type;  // element type mf_rbody reads ("float2", "double", "float")
  size_t smem_bytes = 0;  // dynamic shared memory of the main entry
  // REDUCE kernels: host-evaluated argument struct
  // Prepared input (REDUCE): the kernel reads `prep_cols.size()` columns that
  // a per-dataset pass (entry + "_prep") derives from the source columns.
  enum Prep { PrepNone = 0, PrepF64 = 1, PrepF32 = 2, PrepPair = 3 };
  int prep = PrepNone;
  std::vector<std::vector<std::pair<int, double>>> prep_cols;
  std::vector<int> source_inputs;  // source columns the kernel (or its prep pass) reads
  size_t prep_elem_bytes() const { return prep == PrepF32 ? 4 : 8; }
  bool host_args = false;
  std::vector<Node> nodes;         // the DAG, for host evaluation of the slots
  std::vector<UniformSlot> slots;
  std::vector<int> eval_order;     // parameter-only nodes the slots read, operands first
  int nd = 1, nf = 1;              // array lengths in the struct (>= 1)
  size_t args_bytes() const { return (size_t(nd) * 8 + size_t(nf) * 4 + 7) / 8 * 8; }
  // Fills the argument struct for one parameter vector (params: n_params doubles).
  void fill_args(const double* params, size_t n_params, unsigned char* out) const;
  // The same for `count` parameter vectors (back to back) into `count`
  // argument structs (args_bytes() apart).
  void fill_args_many(const double* params, size_t n_params, size_t count, unsigned char* out) const;
};

// Rewrite of a REDUCE kernel over prepared columns (mf_fold.cpp). When
// `rewritten`, prepared column m is the sum over cols[m] of coefficient x
// source column, and `dag`/`roots` compute the same outputs from the prepared
// columns; `folded` when linearly dependent source columns were merged
// (rank < source_columns).
struct FoldResult {
  bool rewritten = false, folded = false;
  std::vector<std::vector<std::pair<int, double>>> cols;
  std::unique_ptr<Dag> dag;
  std::vector<int> roots;
  int rank = 0, source_columns = 0;
};
// param_defs: per parameter, "" or a parameter-only expression defining it
// from the others (sampled values of defined parameters follow their definition).
FoldResult fold_columns(const Dag& dag, const std::vector<int>& roots,
                        const std::vector<std::string>& param_defs = {});

enum class Elem { F64, F32 };
enum class Kind { Reduce, Store, Generate };

struct GenerateSpec {
  std::vector<std::string> dims;
  std::vector<double> lo, hi;
  double maxprob = 1.0;
};

// Builds the kernel source for the given outputs.
LoweredKernel lower(const std::string& name, Kind kind, Elem elem, const std::vector<std::string>& inputs,
                    const std::vector<std::string>& params, const std::vector<std::string>& exprs,
                    const GenerateSpec* gen = nullptr, bool native_f64 = false, int vec = 0, int block = 0,
                    bool f32_arith = false, bool direct_loads = false, int stages = 0,
                    const std::vector<std::string>& param_defs = {});

// Counts per-event operations of a lowered expression set (diagnostics).
struct OpCount {
  int nodes = 0, per_event = 0, uniform = 0, transcendental = 0, divisions = 0;
};
OpCount count_ops(const std::vector<std::string>& inputs, const std::vector<std::string>& params,
                  const std::vector<std::string>& exprs);

}  // namespace mf

#endif
