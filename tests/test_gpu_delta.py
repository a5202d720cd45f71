"""Delta evaluation through the C ABI (gbofdft_eval_delta): FP32 transforms of
the change of the derived fields against an FP64 reference evaluation, FP64
pointwise terms; compared with full FP64 evaluations (gbofdft_eval) at the
same densities.

Tolerances: FP32 rounding perturbs the convolutions by ~1e-7 of the CHANGE,
so for a smooth density change of relative size eps the energy may differ
from the full FP64 value by 1e-6 eps of the sum of |component energies|.  The
potential may differ by 5e-5 eps of max |V|: the rounding noise of the
transformed change is white, and the von Weizsaecker kernel G^2 amplifies it
up to the grid's cutoff (G^2 ~ 170 bohr^-2 at 0.25 bohr spacing; measured
1.5e-10 at eps = 1e-5 on 128^3).  Both get 1e-12 for FP64 round-off.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def lib():
    from dftpy_gb300 import _lib
    _lib.require_cuda()
    return _lib


def _density(nr, seed=0):
    """A positive density with structure on several scales (2 electrons per
    ~110 bohr^3 on average)."""
    rng = np.random.default_rng(seed)
    x = [np.arange(n) / n for n in nr]
    X, Y, Z = np.meshgrid(*x, indexing="ij")
    r = np.ones(nr)
    for _ in range(6):
        k = rng.integers(1, 5, size=3)
        ph = rng.random(3) * 2 * np.pi
        r += 0.12 * np.cos(2 * np.pi * k[0] * X + ph[0]) * np.cos(2 * np.pi * k[1] * Y + ph[1]) \
            * np.cos(2 * np.pi * k[2] * Z + ph[2])
    return 0.018 * r


def _change(nr, eps, seed=1):
    """A smooth relative change of size eps (a few low Fourier modes)."""
    rng = np.random.default_rng(seed)
    x = [np.arange(n) / n for n in nr]
    X, Y, Z = np.meshgrid(*x, indexing="ij")
    d = np.zeros(nr)
    for _ in range(4):
        k = rng.integers(0, 4, size=3)
        ph = rng.random(3) * 2 * np.pi
        d += np.sin(2 * np.pi * (k[0] * X + k[1] * Y + k[2] * Z) + ph[0])
    return eps * d / np.abs(d).max()


class _Setup:
    def __init__(self, lib, nr, L, wt=True):
        import torch
        self.torch, self.lib = torch, lib
        self.nr = nr
        self.p64 = lib.Plan(nr, L, precision=lib.F64)
        self.p32 = lib.Plan(nr, L, precision=lib.F32)
        self.delta = lib.Delta(self.p64, self.p32)
        rng = np.random.default_rng(5)
        self.vloc = torch.tensor(-0.3 + 0.05 * rng.standard_normal(nr), dtype=torch.float64, device="cuda")
        self.f64 = self._functional(self.p64, torch.float64, wt)
        self.f32 = self._functional(self.p32, torch.float32, wt)

    def _functional(self, plan, dt, wt):
        torch, lib = self.torch, self.lib
        f = lib.Functional()
        f.tf, f.tf_x, f.vw, f.vw_y = 1, 1.0, 1, 1.0
        if wt:
            kern = torch.empty(plan.nr[0], plan.nr[1], plan.n2h, dtype=dt, device="cuda")
            lib.check(lib.load().gbofdft_wt_kernel(plan.handle, 0.018, 1.0, 5 / 6, 5 / 6, lib.ptr(kern),
                                                   lib.stream_ptr()))
            f.wt, f.wt_alpha, f.wt_beta, f.wt_kernel = 1, 5 / 6, 5 / 6, kern.data_ptr()
            setattr(self, "kern_%s" % str(dt)[-2:], kern)
        f.xc, f.hartree = 1, 1
        if dt == torch.float32:
            self.vloc32 = self.vloc.to(torch.float32)
            f.vloc = self.vloc32.data_ptr()
        else:
            f.vloc = self.vloc.data_ptr()
        f.e_ion = 1.5
        return f

    def full(self, rho):
        torch, lib = self.torch, self.lib
        pot = torch.empty_like(rho)
        en = torch.zeros(lib.NE, dtype=torch.float64, device="cuda")
        lib.check(lib.load().gbofdft_eval(self.p64.handle, lib.ptr(rho), self.f64, lib.ptr(pot), lib.ptr(en),
                                          lib.CALC_E | lib.CALC_V, lib.stream_ptr()))
        torch.cuda.synchronize()
        return en.cpu().numpy(), pot.cpu().numpy()

    def delta_eval(self, rho, rebase, calc=None):
        torch, lib = self.torch, self.lib
        pot = torch.empty_like(rho)
        en = torch.zeros(lib.NE, dtype=torch.float64, device="cuda")
        calc = (lib.CALC_E | lib.CALC_V) if calc is None else calc
        lib.check(lib.load().gbofdft_eval_delta(self.delta.handle, lib.ptr(rho), self.f64, self.f32, lib.ptr(pot),
                                                lib.ptr(en), calc, int(rebase), lib.stream_ptr()), "eval_delta")
        torch.cuda.synchronize()
        return en.cpu().numpy(), pot.cpu().numpy()


def _lat(nr):
    return np.diag([0.24 * n + 1.0 for n in nr])


@pytest.mark.parametrize("nr,scale", [((128, 128, 128), 1.0), ((64, 96, 128), 1.0), ((64, 64, 64), 14.0)])
@pytest.mark.parametrize("eps", [1e-5, 1e-3])
def test_delta_matches_full_fp64(lib, nr, scale, eps):
    """scale 14: densities 0.07-0.5, both PZ81 branches (r_s < 1 above
    rho = 0.239) and points whose r_s crosses 1 (the FP64 path at both
    densities)."""
    torch = pytest.importorskip("torch")
    s = _Setup(lib, nr, _lat(nr))
    ra = scale * _density(nr)
    rb = ra * (1.0 + _change(nr, eps))
    rho_a = torch.tensor(ra, dtype=torch.float64, device="cuda")
    rho_b = torch.tensor(rb, dtype=torch.float64, device="cuda")
    # the rebase is the full evaluation
    e_full_a, v_full_a = s.full(rho_a)
    e_a, v_a = s.delta_eval(rho_a, rebase=True)
    np.testing.assert_array_equal(e_a, e_full_a)
    np.testing.assert_array_equal(v_a, v_full_a)
    # a delta evaluation at the reference reproduces it to FP64 round-off
    e_0, v_0 = s.delta_eval(rho_a, rebase=False)
    scale_e = np.abs(e_full_a[:6]).sum()
    assert abs(e_0[-1] - e_full_a[-1]) <= 1e-12 * scale_e
    assert np.abs(v_0 - v_full_a).max() <= 1e-12 * np.abs(v_full_a).max()
    # a moved density: within 1e-6 eps (+ round-off) of the full evaluation
    e_full_b, v_full_b = s.full(rho_b)
    e_b, v_b = s.delta_eval(rho_b, rebase=False)
    tol_e = (1e-6 * eps + 1e-12) * scale_e
    assert np.abs(e_b[:6] - e_full_b[:6]).max() <= tol_e, (e_b - e_full_b, tol_e)
    assert abs(e_b[-1] - e_full_b[-1]) <= tol_e
    vmax = np.abs(v_full_b).max()
    assert np.abs(v_b - v_full_b).max() <= (5e-5 * eps + 1e-12) * vmax
    # the change itself is resolved: the delta result tracks the full one
    # far better than an FP32 evaluation could (1e-7 of E)
    assert abs((e_b[-1] - e_a[-1]) - (e_full_b[-1] - e_full_a[-1])) <= tol_e


def test_delta_potential_only_and_errors(lib):
    torch = pytest.importorskip("torch")
    nr = (64, 64, 64)
    s = _Setup(lib, nr, _lat(nr))
    ra = _density(nr, seed=3)
    rho_a = torch.tensor(ra, dtype=torch.float64, device="cuda")
    rho_b = torch.tensor(ra * (1.0 + _change(nr, 1e-4, seed=4)), dtype=torch.float64, device="cuda")
    # no reference yet
    with pytest.raises(ValueError, match="no reference"):
        s.delta_eval(rho_b, rebase=False)
    s.delta_eval(rho_a, rebase=True)
    _, v_full = s.full(rho_b)
    _, v = s.delta_eval(rho_b, rebase=False, calc=lib.CALC_V)
    assert np.abs(v - v_full).max() <= (5e-5 * 1e-4 + 1e-12) * np.abs(v_full).max()
    # other functional terms than the reference's
    f2 = lib.Functional()
    f2.tf, f2.tf_x, f2.xc, f2.hartree = 1, 1.0, 1, 1
    pot = torch.empty_like(rho_b)
    rc = lib.load().gbofdft_eval_delta(s.delta.handle, lib.ptr(rho_b), f2, None, lib.ptr(pot), None, lib.CALC_V, 0,
                                       lib.stream_ptr())
    assert rc != 0
    assert "differ" in lib.last_error()


def test_delta_create_rejects_unspecialised_grid(lib):
    p64 = lib.Plan((30, 30, 30), _lat((30, 30, 30)), precision=lib.F64)
    p32 = lib.Plan((30, 30, 30), _lat((30, 30, 30)), precision=lib.F32)
    with pytest.raises(ValueError, match="specialisation"):
        lib.Delta(p64, p32)
    q32 = lib.Plan((64, 64, 64), _lat((64, 64, 64)), precision=lib.F32)
    with pytest.raises(ValueError, match="different grids"):
        lib.Delta(p64, q32)


def test_wgc_delta_matches_full_fp64(lib):
    """The WGC term (second-order density-dependent kernel, alpha != beta, six
    transformed fields) as a delta evaluation: the rebase keeps its X / Y
    fields, potential and energy; a delta evaluation at the reference repeats
    the full result, and at a moved density it matches a full FP64
    evaluation within the tolerances above."""
    torch = pytest.importorskip("torch")
    from dftpy_gb300 import batch, systems
    from dftpy_gb300.field import DirectField
    st = systems.fcc_supercell((2, 2, 2), sigma=0.15, seed=4, nr=(64, 64, 64), mg_fraction=0.25, name="wgc_delta")
    total, rho_u = batch.build_evaluator(st, kedf="WGC")
    grid = rho_u.grid
    mean = st.nelec / st.volume
    base = _density(st.nr, seed=7)
    ra = base * (mean / base.mean())
    for eps in (1e-5, 1e-3):
        rb = ra * (1.0 + _change(st.nr, eps, seed=8))
        rho_a = torch.tensor(ra, dtype=torch.float64, device="cuda")
        rho_b = torch.tensor(rb, dtype=torch.float64, device="cuda")
        f64 = total.spec(DirectField(grid, data=rho_a)).ctypes()
        f32 = total.spec(DirectField(grid, data=rho_a.to(torch.float32))).ctypes()
        assert f64.wgc and f32.wgc
        delta = lib.Delta(grid.plan(torch.float64), grid.plan(torch.float32))

        def run(rho, rebase=None):
            pot = torch.empty_like(rho)
            en = torch.zeros(lib.NE, dtype=torch.float64, device="cuda")
            if rebase is None:
                lib.check(lib.load().gbofdft_eval(grid.plan(torch.float64).handle, lib.ptr(rho), f64, lib.ptr(pot),
                                                  lib.ptr(en), lib.CALC_E | lib.CALC_V, lib.stream_ptr()))
            else:
                lib.check(lib.load().gbofdft_eval_delta(delta.handle, lib.ptr(rho), f64, f32, lib.ptr(pot),
                                                        lib.ptr(en), lib.CALC_E | lib.CALC_V, int(rebase),
                                                        lib.stream_ptr()), "eval_delta")
            torch.cuda.synchronize()
            return en.cpu().numpy(), pot.cpu().numpy()

        e_a, v_a = run(rho_a, rebase=True)          # full evaluation, kept as the reference
        e_0, v_0 = run(rho_a, rebase=False)
        e_b, v_b = run(rho_b, rebase=False)
        e_fb, v_fb = run(rho_b)                     # full FP64 (overwrites the reference's fields)
        e_fa, v_fa = run(rho_a)
        np.testing.assert_array_equal(e_a, e_fa)
        np.testing.assert_array_equal(v_a, v_fa)
        scale_e = np.abs(e_fa[:6]).sum()
        assert abs(e_0[-1] - e_fa[-1]) <= 1e-12 * scale_e
        assert np.abs(v_0 - v_fa).max() <= 1e-12 * np.abs(v_fa).max()
        tol_e = (1e-6 * eps + 1e-12) * scale_e
        assert np.abs(e_b[:6] - e_fb[:6]).max() <= tol_e, (eps, e_b - e_fb, tol_e)
        assert abs(e_b[-1] - e_fb[-1]) <= tol_e
        assert np.abs(v_b - v_fb).max() <= (5e-5 * eps + 1e-12) * np.abs(v_fb).max(), eps
        assert abs((e_b[-1] - e_a[-1]) - (e_fb[-1] - e_fa[-1])) <= tol_e
