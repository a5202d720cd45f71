"""Host-side checks that need no GPU: the C ABI library loads and exports every
entry point ``include/gbofdft.h`` declares, the host line search behind the
ABI reproduces the reference's trial sequences, and the host-built tables
match their definitions."""
import ctypes
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _header_symbols():
    txt = open(os.path.join(ROOT, "include", "gbofdft.h")).read()
    return sorted(set(re.findall(r"^int\s+(gbofdft_\w+)\s*\(", txt, flags=re.M)))


@pytest.fixture(scope="module")
def lib():
    from dftpy_gb300 import build
    build.build()
    from dftpy_gb300 import _lib
    return _lib


def test_exports_every_declared_symbol(lib):
    L = lib.load()
    declared = _header_symbols()
    assert len(declared) >= 15
    for name in declared:
        assert hasattr(L, name), name
    assert sorted(lib.EXPORTED) == declared, "ctypes signatures must cover exactly the header"
    assert L.gbofdft_version() == 1


def test_error_path_without_device_work(lib):
    L = lib.load()
    out = ctypes.c_void_p()
    bad = (ctypes.c_int * 3)(0, 4, 4)
    lat = (ctypes.c_double * 9)(1, 0, 0, 0, 1, 0, 0, 0, 1)
    rc = L.gbofdft_plan_create(bad, lat, 1, 0, ctypes.byref(out))
    assert rc == 1 and "nr[0]" in lib.last_error()
    with pytest.raises(ValueError):
        lib.check(rc)


def test_allocation_failure_retried_once(lib):
    """An allocation status makes ``check_alloc`` release PyTorch's cache and
    call once more; a second failure (or any other status) raises."""
    rcs = [4, 0]
    lib.check_alloc(lambda: rcs.pop(0), "create")
    assert rcs == []
    rcs = [4, 4, 0]
    with pytest.raises(MemoryError):
        lib.check_alloc(lambda: rcs.pop(0), "create")
    assert rcs == [0]
    rcs = [1, 0]
    with pytest.raises(ValueError):
        lib.check_alloc(lambda: rcs.pop(0), "create")
    assert rcs == [0]


LS_CASES = {
    "quad": lambda a: ((a - 0.7) ** 2, 2.0 * (a - 0.7)),
    "cos": lambda a: (-np.cos(a - 0.3) + 0.01 * a ** 4, np.sin(a - 0.3) + 0.04 * a ** 3),
    "steep": lambda a: (np.exp(-3.0 * a) + 3.0 * a * a, -3.0 * np.exp(-3.0 * a) + 6.0 * a),
    "flat": lambda a: (-a / (1.0 + 40.0 * a * a), -(1.0 - 40.0 * a * a) / (1.0 + 40.0 * a * a) ** 2),
    "mt1": lambda a: (-a / (a * a + 2.0), (a * a - 2.0) / (a * a + 2.0) ** 2),
}
TASKS = {2: "CONVERGENCE", 3: "WARNING", 4: "ERROR"}


@pytest.mark.parametrize("name", sorted(LS_CASES))
@pytest.mark.parametrize("a0", [0.1, 1e-3, 1.5])
def test_native_line_search_matches_reference(lib, golden, name, a0):
    """gbofdft_dcsrch driven like LineSearchDcsrch2 gives the reference's trials."""
    L = lib.load()
    d = golden("dcsrch")
    fn = LS_CASES[name]
    state = (ctypes.c_double * 32)(1e-4, 0.2, 1e-12, 0.0, np.pi)
    stp = ctypes.c_double(a0)
    f, g = fn(0.0)
    task = 0
    trials = []
    for _ in range(30):
        task = L.gbofdft_dcsrch(state, 32, ctypes.byref(stp), float(f), float(g), task)
        if task != 1:
            break
        trials.append(stp.value)
        f, g = fn(stp.value)
    key = "%s_%g" % (name, a0)
    np.testing.assert_array_equal(np.array(trials), d[key + "_trials"])
    assert str(d[key + "_task"]).startswith(TASKS[task])


def test_host_spline_matches_fitpack():
    from scipy.interpolate import splev, splrep
    from dftpy_gb300._tables import spline_notaknot
    from dftpy_gb300 import systems
    gp, vp = systems.analytic_pp_table(2.0, 1.2)
    x, c = spline_notaknot(gp[1:], vp[1:])
    q = np.random.default_rng(4).uniform(gp[1], gp[-1] * 0.999, 5000)
    i = np.searchsorted(x, q, side="right") - 1
    u = q - x[i]
    val = c[i, 0] + u * (c[i, 1] + u * (c[i, 2] + u * c[i, 3]))
    ref = splev(q, splrep(gp[1:], vp[1:]))
    assert np.max(np.abs(val - ref) / np.abs(ref)) < 1e-12


def test_pme_bm_table():
    from dftpy_gb300._tables import pme_bm
    from oracle import ofdft as O
    nr = (12, 10, 16)
    g = O.Grid(np.eye(3) * 5.0, nr)
    B = O.bspline_barray(g, 10)
    bm = pme_bm(nr, 10)
    b0, b1, b2 = bm[:12], bm[12:22], bm[22:]
    np.testing.assert_allclose(np.einsum("i,j,k->ijk", b0, b1, b2), B, rtol=1e-13, atol=0)


@pytest.mark.parametrize("kind", ["uniform", "log", "short"])
def test_host_spline_grids(kind):
    """Not-a-knot spline on the grids the tables use (uniform eta grids
    included, where the end rows degenerate for a naive elimination)."""
    from scipy.interpolate import splev, splrep
    from dftpy_gb300._tables import lindhard, spline_notaknot, spline_values_deriv
    if kind == "uniform":
        x = np.linspace(0, 50, 50000)
        y = lindhard(x, 1.0, 1.0)
    elif kind == "log":
        x = np.logspace(-5, np.log10(52), 50000)
        y = lindhard(x, 1.0, 1.0)
    else:
        x = np.linspace(0.0, 1.0, 6)
        y = np.sin(3 * x)
    xs, c = spline_notaknot(x, y)
    tck = splrep(x, y)
    u = np.random.default_rng(1).uniform(x[0], x[-1], 20000)
    i = np.clip(np.searchsorted(xs, u, side="right") - 1, 0, xs.size - 2)
    t = u - xs[i]
    v = c[i, 0] + t * (c[i, 1] + t * (c[i, 2] + t * c[i, 3]))
    ref = splev(u, tck)
    assert np.max(np.abs(v - ref)) <= 1e-12 * max(1.0, np.abs(ref).max())
    d = spline_values_deriv(xs, c)
    dref = splev(x, tck, der=1)
    assert np.max(np.abs(d - dref)) <= 1e-9 * max(1.0, np.abs(dref).max())
