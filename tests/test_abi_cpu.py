"""C-ABI checks that need no GPU: the library loads and exports every entry
point the headers declare, and the OPS / GCGSolver layouts match the
reference's (so reference-side code can fill and read them)."""
import ctypes
import os
import re
import shutil
import subprocess

import pytest

import gcge_gb300 as G

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INC = os.path.join(ROOT, "include")


def header_functions():
    names = set()
    for h in ("gcge_ops.h", "gcge_cuda.h"):
        txt = open(os.path.join(INC, h)).read()
        txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
        txt = re.sub(r"typedef struct OPS_ \{.*?\} OPS;", "", txt, flags=re.S)
        txt = re.sub(r"typedef struct GCGSolver_ \{.*?\} GCGSolver;", "", txt, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b([A-Za-z_]\w*)\s*\(", txt, re.M):
            name = m.group(1)
            if name not in ("if", "while", "sizeof", "defined"):
                names.add(name)
    return sorted(names)


@pytest.fixture(scope="module")
def lib():
    if not os.path.exists(G.lib_path()):
        from gcge_gb300.build import build
        build()
    return G.load()


def test_every_declared_symbol_is_exported(lib):
    declared = header_functions()
    assert len(declared) >= 30
    missing = [n for n in declared if not hasattr(lib, n)]
    assert missing == []
    assert set(declared) <= set(G.EXPORTED_SYMBOLS) | {"OPS_Create", "OPS_Setup", "OPS_Destroy"}


def test_status_strings(lib):
    f = lib.ops_cuda_error_string
    f.restype = ctypes.c_char_p
    assert f(0) == b"ok"
    assert b"converged" in f(6)


def test_ops_create_and_cuda_set_without_gpu(lib):
    ops = ctypes.POINTER(G.OPSStruct)()
    lib.OPS_Create(ctypes.byref(ops))
    lib.OPS_CUDA_Set(ops)
    lib.OPS_Setup(ops)
    o = ops.contents
    for slot in ("MatDotMultiVec", "MultiVecAxpby", "MultiVecLinearComb", "MultiVecInnerProd",
                 "MultiVecQtAP", "MultiVecCreateByMat", "MultiVecDestroy", "Printf", "GetWtime"):
        assert getattr(o, slot), slot
    assert o.MatAxpby is None and o.EigenSolver is None
    lib.OPS_Destroy(ctypes.byref(ops))


def test_orth_setup_installs_multivec_orth_without_gpu(lib):
    """MultiVecOrthSetup_* (src/ops_orth.c:395-414, :625-641) fill
    ops->MultiVecOrth and ops->orth_workspace; each ops keeps its own
    setting, and OPS_Destroy releases it.  No device work happens here."""
    a, b = ctypes.POINTER(G.OPSStruct)(), ctypes.POINTER(G.OPSStruct)()
    for ops in (a, b):
        lib.OPS_Create(ctypes.byref(ops))
        lib.OPS_CUDA_Set(ops)
        assert not ops.contents.MultiVecOrth and not ops.contents.orth_workspace
    lib.MultiVecOrthSetup_BinaryGramSchmidt(ctypes.c_int(-1), ctypes.c_int(2),
                                            ctypes.c_double(4.4e-16), None, None, a)
    lib.MultiVecOrthSetup_ModifiedGramSchmidt(ctypes.c_int(-1), ctypes.c_int(2),
                                              ctypes.c_double(4.4e-16), None, None, b)
    assert a.contents.MultiVecOrth and b.contents.MultiVecOrth
    assert a.contents.orth_workspace and a.contents.orth_workspace != b.contents.orth_workspace
    assert lib.ops_cuda_last_error() == 0
    for ops in (a, b):
        lib.OPS_Destroy(ctypes.byref(ops))


def test_command_line_setter_before_setup_is_an_error(lib):
    ops = ctypes.POINTER(G.OPSStruct)()
    lib.OPS_Create(ctypes.byref(ops))
    lib.OPS_CUDA_Set(ops)
    argv = (ctypes.c_char_p * 2)(b"-gcge_compW_cg_order", b"2")
    lib.EigenSolverSetParametersFromCommandLine_GCG(2, argv, ops)
    assert lib.ops_cuda_last_error() == G.GCGE_ERR_ARG
    lib.OPS_Destroy(ctypes.byref(ops))


LAYOUT_PROBE = r"""
#include <stdio.h>
#include <stddef.h>
#include HEADER
int main(void) {
    printf("%zu %zu %zu %zu %zu %zu %zu %zu\n", sizeof(OPS), offsetof(OPS, MultiVecQtAP),
           offsetof(OPS, EigenSolver), offsetof(OPS, app_ops), sizeof(GCGSolver),
           offsetof(GCGSolver, numIter), offsetof(GCGSolver, compW_cg_tol_type),
           offsetof(GCGSolver, compRR_tol));
    return 0;
}
"""


def _probe(tmp_path, header, incs):
    src = tmp_path / "probe.c"
    src.write_text(LAYOUT_PROBE.replace("HEADER", header))
    exe = tmp_path / "probe"
    cmd = ["gcc", "-w", str(src), "-o", str(exe)] + [f"-I{d}" for d in incs]
    subprocess.run(cmd, check=True, capture_output=True)
    return subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split()


@pytest.mark.skipif(shutil.which("gcc") is None, reason="gcc not available")
def test_layout_matches_reference_headers(tmp_path):
    ours = _probe(tmp_path, '"gcge_ops.h"', [INC])
    assert int(ours[0]) == 46 * 8 and int(ours[3]) == 45 * 8
    from oracle.ref_lib import reference_dir
    ref_dir = reference_dir()
    if ref_dir is None:
        pytest.skip("reference headers not present here")
    ref = _probe(tmp_path, '"ops_eig_sol_gcg.h"',
                 [os.path.join(ROOT, "oracle", "ref"), os.path.join(ref_dir, "src"),
                  os.path.join(ref_dir, "app")])
    assert ours == ref


@pytest.mark.skipif(shutil.which("gcc") is None, reason="gcc not available")
def test_request_and_info_layout_match_the_python_mirror(tmp_path):
    """gcge_request / gcge_solve_info as the C header lays them out == the ctypes
    structures the Python mirror passes across the ABI."""
    src = tmp_path / "probe_req.c"
    src.write_text(r'''
#include <stdio.h>
#include <stddef.h>
#include "gcge_cuda.h"
int main(void) {
    printf("%zu %zu %zu %zu %zu %zu\n", sizeof(gcge_request), offsetof(gcge_request, info),
           offsetof(gcge_request, status), offsetof(gcge_request, t_end),
           sizeof(gcge_solve_info), offsetof(gcge_solve_info, pcg_kernel_bytes));
    return 0;
}
''')
    exe = tmp_path / "probe_req"
    subprocess.run(["gcc", "-w", str(src), "-o", str(exe), f"-I{INC}"], check=True,
                   capture_output=True)
    c = [int(x) for x in subprocess.run([str(exe)], check=True, capture_output=True,
                                        text=True).stdout.split()]
    py = [ctypes.sizeof(G.Request), G.Request.info.offset, G.Request.status.offset,
          G.Request.t_end.offset, ctypes.sizeof(G.SolveInfo), G.SolveInfo.pcg_kernel_bytes.offset]
    assert c == py


def test_spmm_tuner_candidates_without_gpu(lib):
    """The tuner's candidate splits (host logic of gcge_gb300/csrc/spmm.cu):
    p launches of ceil(k / p) columns for p from ceil(k / 40) up while a launch
    keeps 8 columns, one p per register width (4, 8, 16, 24, 32, 40)."""
    def width(c):
        return next(w for w in (4, 8, 16, 24, 32, 40) if c <= w)

    def rule(k):
        out, last, p = [], None, -(-k // 40)
        while True:
            c = -(-k // p)
            if out and c < 8:
                return out
            if width(c) != last:
                out.append(c)
                last = width(c)
            if c <= 8:
                return out
            p += 1

    for k in list(range(1, 130)) + [200, 320, 400]:
        got = G.spmm_tune_candidates(k)
        assert got == rule(k), k
        assert all(1 <= c <= 40 for c in got) and got == sorted(got, reverse=True)
        # every split covers the k columns with at most 40 per launch
        assert -(-k // got[0]) == -(-k // 40)
    assert G.spmm_tune_candidates(40) == [40, 20, 14, 8]
    cnt = ctypes.c_int()
    assert lib.GCGE_SpMMTuneCandidates(0, None, 0, ctypes.byref(cnt)) == G.GCGE_ERR_ARG
    assert lib.ops_cuda_last_error() == G.GCGE_ERR_ARG
    assert lib.GCGE_SetSpMMTuning(0) == G.GCGE_OK


# The C examples of INTEGRATION.md, each compiled as a function body against
# the headers and linked against the library (not run: no device here).
_SNIPPET_PRELUDES = {
    "## 1. Drop-in": "void snippet(int n, int *j_col, int *i_row, double *data, int nevMax, "
                     "int nevGiven, double *x0, int block_size, int nevInit, double gapMin, "
                     "int maxit, int nev, double *eval, double *evec_host)",
    "## 1b.": "void snippet(OPS *ops, int argc, char **argv)",
    "## 2d.": "void snippet(OPS *ops, int L, int *n, int **a_col, int **a_row, double **a_val, "
              "int **p_col, int **p_row, double **p_val, int block_size, int *max_iter, "
              "double *rate, double *tol, double *dbl_ws, int *int_ws, void **b, void **x, "
              "int *start, int *end)",
}


def _integration_snippets():
    text = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    out = {}
    for head, proto in _SNIPPET_PRELUDES.items():
        sec = text[text.index(head):]
        body = sec[sec.index("```c\n") + 5:]
        body = body[:body.index("```")]
        out[head] = (proto, "\n".join(l for l in body.splitlines()
                                      if not l.startswith("#include")))
    return out


@pytest.mark.skipif(shutil.which("gcc") is None, reason="gcc not available")
@pytest.mark.parametrize("head", list(_SNIPPET_PRELUDES))
def test_integration_examples_compile_and_link(lib, tmp_path, head):
    proto, body = _integration_snippets()[head]
    src = tmp_path / "snippet.c"
    src.write_text("#include <stdlib.h>\n#include \"gcge_cuda.h\"\n" + proto +
                   " {\n    int l, i;\n    (void)l; (void)i;\n" + body +
                   "\n}\nint main(void) { return 0; }\n")
    libdir = os.path.dirname(G.lib_path())
    r = subprocess.run(["gcc", "-std=c99", "-Wall", "-Wno-unused-variable",
                        "-Wno-unused-but-set-variable", "-I" + INC, str(src), "-o",
                        str(tmp_path / "snippet"), "-L" + libdir, "-lgcge_cuda"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
