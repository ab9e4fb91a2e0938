"""Block AMG without a GPU: the CPU restatement of the reference's BlockAMG
(oracle/amg_oracle.py, src/ops_lin_sol.c:466-715) against the fixtures the
compiled reference made (tests/golden/make_golden_amg.py) and against a live
reference run where it is built; the hierarchy generator; and the C-ABI
surface of the library's BlockAMG (setup, layout of the solver record, the
argument checks that run before any device work)."""
import ctypes
import json
import os
import shutil
import subprocess

import numpy as np
import pytest

import gcge_gb300 as G
from gcge_gb300 import problems as P
from oracle.amg_oracle import block_amg, block_pcg

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")
INC = os.path.join(os.path.dirname(HERE), "include")


def load_cases():
    import sys
    if GOLDEN not in sys.path:
        sys.path.insert(0, GOLDEN)
    import make_golden_amg
    with open(os.path.join(GOLDEN, "golden_amg.json")) as f:
        meta = json.load(f)
    return make_golden_amg, meta, dict(np.load(os.path.join(GOLDEN, "golden_amg.npz")))


def run_oracle(mg, c):
    A, T, b, x0 = mg.inputs(c)
    x = np.array(x0, order="F", copy=True)
    res, cycles = block_amg([a.to_scipy() for a in A], [t.to_scipy() for t in T], b, x,
                            c["max_iter"], c["rate"], c["tol"], c["tol_type"])
    return A, b, x, res, cycles


@pytest.mark.parametrize("name", ["lap2d_63_L3_fixed", "lap2d_63_L3_abs", "lap2d_127_L4_rel",
                                  "lap2d_31_L2_wide"])
def test_oracle_matches_reference_fixture(name):
    mg, meta, xs = load_cases()
    c = meta[name]
    A, b, x, res, cycles = run_oracle(mg, c)
    xr = xs[name]
    assert x.shape == xr.shape
    assert np.abs(x - xr).max() <= 1e-12 * np.abs(xr).max()
    # the residual field is an absolute residual norm, formed by cancellation
    bn = np.linalg.norm(b, axis=0).max()
    assert abs(res - c["residual"]) <= 1e-6 * abs(c["residual"]) + 1e-13 * bn
    assert 1 <= cycles <= c["max_iter"][0]
    if c["tol"][0] > 0 and cycles < c["max_iter"][0]:
        assert res < c["tol"][0]


def test_oracle_matches_live_reference():
    from oracle import ref_lib
    if not ref_lib.available():
        pytest.skip("compiled reference not built here")
    A, T = P.multigrid_2d(31, 63, 3)  # 31 x 63 -> 15 x 31 -> 7 x 15
    n, k = A[0].n, 5
    b = (P.splitmix_uniform(21, n * k, 0) - 0.5).reshape((n, k), order="F")
    x0 = (P.splitmix_uniform(21, n * k, 1) - 0.5).reshape((n, k), order="F")
    for tol_type, tol in (("abs", [1e-8, 1e-11, 1e-11]), ("rel", [1e-9] * 3)):
        mi, rate = [10, 3, 2, 2, 3, 15], [1e-1, 1e-2, 1e-3]
        xr, rr = ref_lib.ref_block_amg(A, T, b, x0, mi, rate, tol, tol_type)
        x = np.array(x0, order="F", copy=True)
        res, _ = block_amg([a.to_scipy() for a in A], [t.to_scipy() for t in T], b, x, mi, rate,
                           tol, tol_type)
        assert np.abs(x - xr).max() <= 1e-12 * np.abs(xr).max()
        assert abs(res - rr) <= 1e-6 * abs(rr) + 1e-13 * np.linalg.norm(b)


def test_block_pcg_residual_field_names_the_first_column_of_the_last_step():
    """The residual field of BlockPCG (src/ops_lin_sol.c:406-410) is the last
    residual of the first column in the compacted int_ws list: column 0 (an
    eigenvector, converged after one step) has left, so the field is column
    1's, as a solve of column 1 alone reports it."""
    nx = 20
    A = P.laplace2d(nx, nx).to_scipy()
    n = A.shape[0]
    s = np.sin(np.pi * np.arange(1, nx + 1) / (nx + 1))
    b = np.zeros((n, 2), order="F")
    b[:, 0] = np.kron(s, s)
    b[:, 1] = P.splitmix_uniform(5, n, 0)
    x = np.zeros((n, 2), order="F")
    st = block_pcg(lambda v: A @ v, b, x, 200, 0.0, 1e-12, "abs")
    x1 = np.zeros((n, 1), order="F")
    st1 = block_pcg(lambda v: A @ v, np.asfortranarray(b[:, 1:]), x1, 200, 0.0, 1e-12, "abs")
    assert st.niter == st1.niter > 2
    assert st.residual == pytest.approx(st1.residual, rel=1e-6)
    assert 1e-14 < st.residual <= 1e-12


def test_multigrid_hierarchy_is_galerkin_and_exact():
    A, T = P.multigrid_2d(31, 15, 3)
    assert [a.n for a in A] == [31 * 15, 15 * 7, 7 * 3]
    for l, t in enumerate(T):
        assert (t.nrows, t.ncols) == (A[l].n, A[l + 1].n)
        Ps = t.to_scipy()
        ref = (Ps.T @ A[l].to_scipy() @ Ps).toarray()
        assert np.array_equal(A[l + 1].to_scipy().toarray(), ref)   # dyadic: exact
        assert np.array_equal(t.transpose().to_scipy().toarray(), Ps.T.toarray())
    with pytest.raises(ValueError):
        P.multigrid_2d(32, 31, 2)


# ----------------------------------------------------------------- C ABI
def _zero_handles(count):
    """Host buffers that no CUDA handle check accepts (zero magic)."""
    bufs = [(ctypes.c_uint64 * 8)() for _ in range(count)]
    return bufs, [ctypes.c_void_p(ctypes.addressof(b)) for b in bufs]


@pytest.fixture(scope="module")
def lib():
    if not os.path.exists(G.lib_path()):
        from gcge_gb300.build import build
        build()
    return G.load()


def test_setup_installs_block_amg_with_the_reference_record(lib):
    ops = ctypes.POINTER(G.OPSStruct)()
    lib.OPS_Create(ctypes.byref(ops))
    lib.OPS_CUDA_Set(ops)
    lib.OPS_Setup(ops)
    lib.ops_cuda_last_error()                            # clear what earlier calls left
    try:
        assert ops.contents.MultiVecFromItoJ              # installed by OPS_CUDA_Set
        keep, h = _zero_handles(3 + 2 + 15 + 2)
        mats, trans, ws = h[:3], h[3:5], [h[5 + 3 * i:8 + 3 * i] for i in range(5)]
        arr = G.AMGArrays(mats, trans, ws, [4, 2, 2, 3, 3, 9], [0.1, 0.2, 0.3],
                          [1e-8, 1e-9, 1e-10], 6)
        arr.setup(lib, ops, "rel")
        assert lib.ops_cuda_last_error() == G.GCGE_OK
        rec = ctypes.cast(ops.contents.multi_linear_solver_workspace,
                          ctypes.POINTER(G.BlockAMGSolver)).contents
        assert rec.num_levels == 3 and rec.tol_type == b"rel" and rec.residual == -1.0
        assert rec.max_iter == ctypes.addressof(arr.max_iter)
        assert rec.A_array == ctypes.addressof(arr.A) and rec.P_array == ctypes.addressof(arr.P)
        assert [rec.mv_array_ws[i] for i in range(5)] == [ctypes.addressof(a) for a in arr.levels]
        # the installed solver checks the hierarchy before any device work
        fn = ctypes.cast(ops.contents.MultiLinearSolver, G._LINSOL)
        fn(h[0], h[20], h[21], G._I2(0, 0), G._I2(6, 6), ctypes.cast(ops, ctypes.c_void_p))
        assert lib.ops_cuda_last_error() == 4            # GCGE_ERR_HANDLE: not a CUDA matrix
        fn(h[0], h[20], h[21], G._I2(0, 1), G._I2(6, 6), ctypes.cast(ops, ctypes.c_void_p))
        assert lib.ops_cuda_last_error() == G.GCGE_ERR_ARG
        # the transfer slot rejects foreign handles the same way
        slot = ctypes.cast(ops.contents.MultiVecFromItoJ, G._FT["MultiVecFromItoJ"])
        slot(arr.P, 0, 1, h[20], h[21], G._I2(0, 0), G._I2(2, 2), None,
             ctypes.cast(ops, ctypes.c_void_p))
        assert lib.ops_cuda_last_error() == 4
    finally:
        lib.OPS_Destroy(ctypes.byref(ops))


def test_transfer_creation_checks_indices_on_the_host(lib):
    h = ctypes.c_void_p()
    cp = np.array([0, 2, 3], dtype=np.int32)
    ri = np.array([0, 5, 1], dtype=np.int32)             # row 5 of a 3-row P
    va = np.ones(3)
    st = lib.CUDA_TransferCreateFromCCS(ctypes.byref(h), 3, 2, cp.ctypes.data_as(ctypes.c_void_p),
                                        ri.ctypes.data_as(ctypes.c_void_p),
                                        va.ctypes.data_as(ctypes.c_void_p))
    assert st == G.GCGE_ERR_ARG and not h.value
    cp_bad = np.array([0, 2, 1], dtype=np.int32)         # decreasing column pointers
    st = lib.CUDA_TransferCreateFromCCS(ctypes.byref(h), 3, 2,
                                        cp_bad.ctypes.data_as(ctypes.c_void_p),
                                        ri.ctypes.data_as(ctypes.c_void_p),
                                        va.ctypes.data_as(ctypes.c_void_p))
    assert st == G.GCGE_ERR_ARG


LAYOUT = r"""
#include <stdio.h>
#include <stddef.h>
#include HEADER
int main(void) {
    printf("%zu %zu %zu %zu %zu %zu\n", sizeof(BlockAMGSolver), offsetof(BlockAMGSolver, tol_type),
           offsetof(BlockAMGSolver, num_levels), offsetof(BlockAMGSolver, mv_array_ws),
           offsetof(BlockAMGSolver, niter), offsetof(BlockAMGSolver, residual));
    return 0;
}
"""


def _layout(tmp_path, header, incs):
    src = tmp_path / "amg_layout.c"
    src.write_text(LAYOUT.replace("HEADER", header))
    exe = tmp_path / "amg_layout"
    subprocess.run(["gcc", "-w", str(src), "-o", str(exe)] + [f"-I{d}" for d in incs],
                   check=True, capture_output=True)
    return [int(v) for v in subprocess.run([str(exe)], check=True, capture_output=True,
                                           text=True).stdout.split()]


@pytest.mark.skipif(shutil.which("gcc") is None, reason="gcc not available")
def test_block_amg_record_layout(tmp_path):
    ours = _layout(tmp_path, '"gcge_ops.h"', [INC])
    S = G.BlockAMGSolver
    assert ours == [ctypes.sizeof(S), S.tol_type.offset, S.num_levels.offset,
                    S.mv_array_ws.offset, S.niter.offset, S.residual.offset]
    from oracle.ref_lib import reference_dir
    ref_dir = reference_dir()
    if ref_dir is None:
        pytest.skip("reference headers not present here")
    ref = _layout(tmp_path, '"ops_lin_sol.h"',
                  [os.path.join(os.path.dirname(HERE), "oracle", "ref"),
                   os.path.join(ref_dir, "src"), os.path.join(ref_dir, "app")])
    assert ours == ref
