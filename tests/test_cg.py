"""The solve after assembly: batched conjugate gradient on the cloth system
matrix (lower triangle, as the engine's cloth workload outputs it), checked
against dense NumPy linear algebra."""
import ctypes as C

import numpy as np
import pytest

from symboliclib_gb300 import native


def dense(w, values):
    r, c, cp, ri = w.pattern()
    L = np.zeros((r, c))
    for j in range(c):
        for e in range(cp[j], cp[j + 1]):
            L[ri[e], j] = values[e]
    return L + L.T - np.diag(np.diag(L))


def test_pattern_above_diagonal_is_rejected():
    cp = np.array([0, 2, 3], np.int64)
    ri = np.array([0, 1, 0], np.int32)  # column 1 holds row 0: above the diagonal
    h = C.c_void_p()
    lib = native.symgb()
    assert lib.symgb_cg_create(2, cp.ctypes.data, ri.ctypes.data, 1, 1, C.byref(h)) == -1  # SYMGB_ERR_ARGUMENT
    bad = np.array([0, 1, 5], np.int32)  # row index out of range
    assert lib.symgb_cg_create(2, cp.ctypes.data, bad.ctypes.data, 0, 1, C.byref(h)) == -1


@pytest.mark.gpu
@pytest.mark.parametrize("sets", [1, 3])
def test_multiply_matches_dense(sets):
    torch = pytest.importorskip("torch")
    w = native.Workload("cloth", 8, 5)
    r, c, cp, ri = w.pattern()
    vals = np.stack([w.numeric * (1.0 + 0.1 * s) for s in range(sets)])
    p = np.random.default_rng(1).standard_normal((sets, r))
    cg = native.CG(r, cp, ri, True, sets)
    q = torch.empty((sets, r), dtype=torch.float64, device="cuda")
    cg.multiply(torch.from_numpy(vals).cuda(), torch.from_numpy(p).cuda(), q)
    for s in range(sets):
        ref = dense(w, vals[s]) @ p[s]
        scale = np.abs(dense(w, vals[s])) @ np.abs(p[s])
        assert np.max(np.abs(q[s].cpu().numpy() - ref) / scale) <= 1e-14


@pytest.mark.gpu
@pytest.mark.parametrize("size,sets", [(5, 1), (12, 4)])
def test_solve_matches_dense(size, sets):
    torch = pytest.importorskip("torch")
    w = native.Workload("cloth", size, 11)
    r, c, cp, ri = w.pattern()
    vals = np.stack([w.numeric * (1.0 + 0.05 * s) for s in range(sets)])
    b = np.random.default_rng(2).standard_normal((sets, r))
    cg = native.CG(r, cp, ri, True, sets)
    x = torch.empty((sets, r), dtype=torch.float64, device="cuda")
    it, res = cg.solve(torch.from_numpy(vals).cuda(), torch.from_numpy(b).cuda(), x, tol=1e-12, max_iter=5000)
    assert res <= 1e-12 and 0 < it <= 5000
    for s in range(sets):
        A = dense(w, vals[s])
        xs = x[s].cpu().numpy()
        assert np.linalg.norm(A @ xs - b[s]) <= 1e-11 * np.linalg.norm(b[s])
        ref = np.linalg.solve(A, b[s])
        assert np.linalg.norm(xs - ref) <= 1e-8 * np.linalg.norm(ref)


@pytest.mark.gpu
def test_assembly_then_solve_on_the_device():
    """A assembled by the engine (results left on the device) feeds the solver."""
    torch = pytest.importorskip("torch")
    w = native.Workload("cloth", 10, 3)
    sets = 2
    u = native.Unit.from_workload(w)
    u.set_schedule(kind=native.SCHEDULE_LEVELS, math=native.MATH_FAST)
    u.set_num_sets(sets)
    for i, a in enumerate(w.inputs):
        u.set_arg(i, np.tile(a, sets))
    u.run()
    nnz = len(w.numeric)
    vals = torch.empty((sets, nnz), dtype=torch.float64, device="cuda")
    native.check(native.symgb().symgb_get_result_sets_device(u.handle, C.c_void_p(vals.data_ptr()), 0))
    r, c, cp, ri = w.pattern()
    b = torch.ones((sets, r), dtype=torch.float64, device="cuda")
    x = torch.empty_like(b)
    cg = native.CG(r, cp, ri, True, sets)
    it, res = cg.solve(vals, b, x, tol=1e-11, max_iter=5000)
    assert res <= 1e-11
    A = dense(w, w.numeric)
    assert np.linalg.norm(A @ x[1].cpu().numpy() - 1.0) <= 1e-9 * np.sqrt(r)


@pytest.mark.gpu
def test_iteration_limit_reports_the_residual():
    torch = pytest.importorskip("torch")
    w = native.Workload("cloth", 12, 11)
    r, c, cp, ri = w.pattern()
    cg = native.CG(r, cp, ri, True, 1)
    x = torch.empty((1, r), dtype=torch.float64, device="cuda")
    it, res = cg.solve(torch.from_numpy(w.numeric[None, :].copy()).cuda(), torch.ones((1, r), dtype=torch.float64,
                                                                                       device="cuda"), x, 1e-14, 3)
    assert it == 3 and res > 1e-14
