"""Lowering of the reference's kernel text to CUDA C and its NVRTC compile for sm_103a (CPU only)."""
import pytest

from conftest import kernel_spec, load_golden


def _src(g, name, elem, kind=0, native_f64=False):
    from morefit_gb300.backend import lower_source
    k = kernel_spec(g, name)
    return lower_source(name, kind, elem, k["inputs"], k["params"], k["exprs"], native_f64=native_f64)


def _entry(src, head):
    """Text of one entry point: from its name to the next entry."""
    i = src.index(head)
    j = src.find('extern "C"', i)
    return src[i:] if j < 0 else src[i:j]


def test_shared_subexpressions_evaluated_once():
    from morefit_gb300 import _lib as L
    g = load_golden("pwave_n1000.json")
    src = _src(g, "lh_grad_kernel", L.MF_F64, native_f64=True)
    body = _entry(src, "mf_reduce(")
    # one density, one log and one reciprocal per event (vector width 2)
    assert body.count("= log(") == 2
    assert body.count("__drcp_rn(") == 2
    dw = _src(g, "lh_grad_kernel", L.MF_F64)
    body = _entry(dw, "void MF_BOUNDS mf_reduce(")
    # double-float kernel: two events per thread, one reciprocal each; the
    # NLL output log(p) is summed as the log of a running product (one factor
    # per event, one logarithm per thread)
    assert body.count("mf_dw_log(") == 0 and body.count("mf_dw_rcp(") == 2
    assert body.count("mf_dw_logprod(") == 2 and body.count("mf_dw_logprod_log(") == 1
    assert " log(" not in body
    # the event loop reads the 9 folded basis columns as float pairs
    assert "data + (mf_u64)8 * stride" in body and "data + (mf_u64)9 * stride" not in body
    assert "const float4 l8 = " in body and "mf_dw_split(" not in body


def test_pwave_basis_folds_to_nine_columns():
    """The 11 hoisted angular columns enter the density and every derivative
    only as S9*b3 + ... - Fl*b10 + pb0*(b11 + b12) + Fl*b13: b11 + b12 and
    b10 - b13 are the only combinations the kernels need."""
    from morefit_gb300 import _lib as L
    g = load_golden("pwave_n1000.json")
    for name in ("lh_kernel", "lh_grad_kernel", "lh_hessian_kernel"):
        for elem, native in ((L.MF_F64, False), (L.MF_F64, True), (L.MF_F32, False)):
            src = _src(g, name, elem, native_f64=native)
            assert "// reads 9 prepared columns" in src, (name, elem, native)
            assert "//   y7 = + 1*morefit_eventbuffer_10 + -1*morefit_eventbuffer_13" in src
            assert "//   y8 = + 1*morefit_eventbuffer_11 + 1*morefit_eventbuffer_12" in src
            prep = src[src.index("mf_reduce_prep("):]
            # the prep pass reads the source columns (3..13), never the raw observables
            assert "data + (mf_u64)13 * stride" in prep and "data + (mf_u64)0 * stride" not in prep


def test_mass_kernels_do_not_fold():
    """One observable column: nothing to fold. The double-float kernels still
    read it pre-split; the FP32 kernels read the input buffer directly."""
    from morefit_gb300 import _lib as L
    g = load_golden("mass_n1000.json")
    dw = _src(g, "lh_grad_kernel", L.MF_F64)
    assert "// reads 1 prepared columns (FP64 as float pairs)" in dw
    f32 = _src(g, "lh_grad_kernel", L.MF_F32)
    assert "prepared" not in f32 and "mf_reduce_prep(" not in f32


def test_hessian_kernel_shares_the_density():
    from morefit_gb300 import _lib as L
    g = load_golden("pwave_n1000.json")
    src = _src(g, "lh_hessian_kernel", L.MF_F64, native_f64=True)
    body = _entry(src, "mf_reduce(")
    assert body.count("__drcp_rn(") <= 4  # 1/p and 1/p^2, twice for the two vector lanes


def test_float_kernels_use_float_literals_and_functions():
    from morefit_gb300 import _lib as L
    g = load_golden("mass_n1000.json")
    src = _src(g, "lh_grad_kernel", L.MF_F32)
    body = _entry(src, "mf_reduce(")
    assert "expf(" in body and "logf(" in body
    assert " exp(" not in body and " log(" not in body
    assert "double2" not in body and "float4" in body
    # the NLL-only kernel: the density's dot product with the parameter-only
    # factors compensated, its logarithm summed as a double-float running product
    body = _entry(_src(g, "lh_kernel", L.MF_F32), "mf_reduce(")
    assert "mf_dw_acc_mulfw(" in body and "mf_dw_logprod(" in body and "logf(" not in body
    assert " exp(" not in body and " log(" not in body


@pytest.mark.parametrize("workload", ["pwave", "mass", "mass_w", "cbpoly"])
@pytest.mark.parametrize("elem", [0, 1])
def test_all_kernels_compile_without_spills(workload, elem):
    from morefit_gb300 import _lib as L
    from morefit_gb300.backend import compile_check
    g = load_golden(f"{workload}_n1000.json")
    for k in g["kernels"]:
        gen = None
        if k.get("generate"):
            kind = L.MF_KERNEL_GENERATE
            gen = (k["outputs"], k["lo"], k["hi"], k["maxprob"])
        elif k["name"] == "precompute_kernel":
            kind = L.MF_KERNEL_STORE
        else:
            kind = L.MF_KERNEL_REDUCE
        info = compile_check(k["name"], kind, elem, k["inputs"], k["params"], k["exprs"], gen)
        assert info["registers"] > 0
        # The P-wave kernels (the benchmarked path) never spill; kernels whose
        # double-float body calls an FP64 function (exp in the mass fit) may
        # keep a few bytes of call frame.
        limit = 0 if workload == "pwave" else 64
        assert info["spill_bytes"] <= limit, (k["name"], info)


def test_spwave_kernels_compile_without_spills_in_double_float():
    """S+P wave (14 parameters): every double-float kernel, the 105-output
    Hessian included (partials beyond MF_NREG in shared memory), compiles
    without spilling; in FP32 only the Hessian spills (a Likelihood then
    evaluates it in register-only parts)."""
    from morefit_gb300 import _lib as L
    from morefit_gb300.backend import compile_check
    g = load_golden("spwave_n2000.json")
    for elem in (L.MF_F64, L.MF_F32):
        for k in g["kernels"]:
            gen = None
            if k.get("generate"):
                kind = L.MF_KERNEL_GENERATE
                gen = (k["outputs"], k["lo"], k["hi"], k["maxprob"])
            elif k["name"] == "precompute_kernel":
                kind = L.MF_KERNEL_STORE
            else:
                kind = L.MF_KERNEL_REDUCE
            info = compile_check(k["name"], kind, elem, k["inputs"], k["params"], k["exprs"], gen)
            if elem == L.MF_F64 or k["name"] != "lh_hessian_kernel":
                assert info["spill_bytes"] == 0, (elem, k["name"], info)


def test_parse_error_is_reported():
    from morefit_gb300 import _lib as L
    from morefit_gb300.backend import lower_source
    with pytest.raises(L.MFError, match="PARSE"):
        lower_source("bad", 0, 0, ["x"], [], ["log(x"])
    with pytest.raises(L.MFError, match="PARSE"):
        lower_source("bad", 0, 0, ["x"], [], ["foo(x)"])


def test_spwave_folds_with_parameter_definitions():
    """S+P wave with acceptance: 17 hoisted columns; the density's coefficients
    (1-FS)(1-Fl) (two columns) and +-(1-FS)Fl (two columns) are hoisted parameter
    buffers, so the relations show only when their definitions are given."""
    from morefit_gb300 import _lib as L
    from morefit_gb300.backend import lower_source
    g = load_golden("spwave_n2000.json")
    k = kernel_spec(g, "lh_grad_kernel")
    defs = dict(g["grad_buffers"])
    with_defs = lower_source("g", L.MF_KERNEL_REDUCE, L.MF_F64, k["inputs"], k["params"], k["exprs"],
                             param_defs=[defs.get(p, "") for p in k["params"]])
    assert "// reads 15 prepared columns (FP64 as float pairs) derived from 17 source columns" in with_defs
    without = lower_source("g", L.MF_KERNEL_REDUCE, L.MF_F64, k["inputs"], k["params"], k["exprs"])
    assert "// reads 16 prepared columns" in without


def test_expression_set_matches_single_evaluation():
    """mf_expr_set (parsed once, evaluated per row) gives the values of
    mf_eval_expressions row by row (host only)."""
    import numpy as np
    from morefit_gb300.backend import ExpressionSet, eval_expressions
    g = load_golden("spwave_n2000.json")
    names = g["parameters"]
    exprs = [e for _, e in g["hessian_buffers"]]
    rows = np.array(g["truth"]) * (1.0 + np.random.default_rng(3).uniform(-0.2, 0.2, (7, len(names))))
    got = ExpressionSet(names, exprs).eval(rows)
    for r in range(len(rows)):
        assert np.array_equal(got[r], eval_expressions(names, rows[r], exprs))


@pytest.mark.parametrize("workload", ["pwave", "mass", "spwave"])
@pytest.mark.parametrize("elem", [0, 1])
def test_resident_module_compiles(workload, elem):
    """The resident module of a fit's two synchronous kernels (NLL and
    NLL + gradient): each kernel's per-block work in its own namespace, its
    macros undefined after it, one resident entry; it compiles for sm_103a
    (spills as its kernels do), and each member's work is its
    single-evaluation entry's with blockIdx.x / gridDim.x as parameters."""
    from morefit_gb300 import _lib as L
    from morefit_gb300.backend import compile_check_resident
    g = load_golden(f"{workload}_n1000.json" if workload != "spwave" else "spwave_n2000.json")
    ks = [kernel_spec(g, n) for n in ("lh_kernel", "lh_grad_kernel")]
    info = compile_check_resident([(k["name"], k["inputs"], k["params"], k["exprs"]) for k in ks], elem)
    # as for the kernels themselves: the P-wave never spills; a double-float
    # body that calls an FP64 function (exp in the mass fit) may keep a call frame
    assert info["registers"] > 0 and info["spill_bytes"] <= (0 if workload == "pwave" else 64), info
    src = info["source"]
    assert "namespace mfr0 {" in src and "namespace mfr1 {" in src and "#undef MF_NOUT" in src
    assert src.count('extern "C"') == 1 and "mf_resident(" in src
    body = src[src.index("void mf_rbody("):src.index("}  // namespace mfr0")]
    assert "blockIdx.x" not in body and "gridDim.x" not in body
    single = _entry(_src(g, "lh_kernel", elem), "mf_reduce(")
    assert single.count("__syncthreads()") == body.count("__syncthreads()")


def test_many_output_kernels_keep_partials_in_shared_memory():
    """Double-float kernels of more than 64 outputs keep the per-thread
    partials beyond MF_NREG in shared memory (64-thread blocks) and sum
    outputs x + u as x plus the event count times u; the S+P-wave Hessian then
    compiles without spilling. FP32 kernels and smaller ones keep every partial
    in registers."""
    import re
    from morefit_gb300 import _lib as L
    from morefit_gb300.backend import compile_check, lower_source
    g = load_golden("spwave_n2000.json")
    k = kernel_spec(g, "lh_hessian_kernel")
    defs = dict(g["hessian_buffers"])
    pd = [defs.get(p, "") for p in k["params"]]
    src = lower_source("h", L.MF_KERNEL_REDUCE, L.MF_F64, k["inputs"], k["params"], k["exprs"], param_defs=pd)
    nreg = int(re.search(r"#define MF_NREG (\d+)", src).group(1))
    assert "#define MF_BLOCK 64" in src and nreg < 105 and "mf_sacc[" in src
    assert "mf_cnt++" in src and "(float)mf_cnt" in src
    info = compile_check("h", L.MF_KERNEL_REDUCE, L.MF_F64, k["inputs"], k["params"], k["exprs"], param_defs=pd)
    assert info["spill_bytes"] == 0, info
    f32 = lower_source("h", L.MF_KERNEL_REDUCE, L.MF_F32, k["inputs"], k["params"], k["exprs"], param_defs=pd)
    assert "#define MF_NREG 105" in f32 and "mf_sacc[" not in f32
    pw = load_golden("pwave_n1000.json")
    kp = kernel_spec(pw, "lh_hessian_kernel")
    psrc = lower_source("h", L.MF_KERNEL_REDUCE, L.MF_F64, kp["inputs"], kp["params"], kp["exprs"])
    assert "#define MF_NREG 36" in psrc and "#define MF_BLOCK 256" in psrc and "mf_sacc[" not in psrc
