"""Direct density optimisation (``dftpy/optimization/optimization.py``).

``Optimization(optimization_method="TN", optimization_options=..., EnergyEvaluator=total)``
runs the truncated-Newton solver of the reference on the GPU
(``gbofdft_optimize_tn``): the whole loop -- inner CG with finite-difference
Hessian products, orthogonal rotation, More-Thuente line search, energy
convergence test -- is native code with device-resident fields.

Added option ``precision``: "fp64" (default for float64 densities, the
reference's arithmetic), "fp32", or "mixed" (FP32 fields and transforms until
the FP32 energy stops resolving progress, then FP64 iterations from that
density to the requested ``econv``).  Reductions are FP64 in every mode.
In the FP64 refinement of "mixed", ``refine="split"`` (default) evaluates
the Hessian-vector products of the inner CG loop in FP32
(``gbofdft_optimize_tn_split``) and stops once the model decrease of the next
Newton step is below ``refine_pred_stop`` (default econv / 100: the model
decrease measures the density error, and forces need it that small);
``refine="fp64"`` runs the plain FP64 TN to ``econv``.
"""
import ctypes
import time

import numpy as np
import torch

from . import _lib, torch_ops
from .field import DirectField
from .functional.output import FunctionalOutput
from .functional.total_functional import TotalFunctional

DEFAULTS = {
    "maxcor": 6,
    "ftol": 1.0e-7,
    "xtol": 1.0e-12,
    "maxfun": 50,
    "maxiter": 200,
    "maxls": 30,
    "econv": 1.0e-5,
    "c1": 1e-4,
    "c2": 0.2,
    "algorithm": "EMM",
    "vector": "Orthogonalization",
    "ncheck": 2,
    "precision": None,
    "eps": None,
    "fp32_econv": None,
    "fp32_eps": -1.0e-3,
    "refine_maxls": 10,
    "refine": "split",
    # refinements that end in a line-search failure while the energy still
    # moved by more than econv are started again from their last density
    # this many times (the 4000-atom LMGP solve ends the same either way: its
    # restart stops after one step at the same energy)
    "refine_restarts": 0,
    # > 0: the TN returns at once with converged = 3 (density unchanged) when
    # the residual norm at the start is above it -- a caller's check of a
    # starting density without an evaluation of its own (no reference
    # counterpart)
    "start_residual_max": 0.0,
    "refine_pred_stop": None,
    # relative energy resolution of the evaluations, for the line-search
    # acceptance on the derivative (mixed precision only): the PZ81 LDA is
    # discontinuous at r_s = 1, which makes E(theta) jump by ~1e-10 |E| over
    # tiny steps in FP64; FP32 fields add their own rounding
    "refine_eres": 3e-10,
    "fp32_eres": 1e-7,
    # energy-change checks per stage of "mixed": a stage ends after one
    # accepted step below its threshold (its next direction would be
    # discarded by the model-decrease stop)
    "stage_ncheck": 1,
    # the refinement stops on the Newton model decrease (refine_pred_stop),
    # which measures the density error; energy changes at FP64 resolution
    # are noisy (see refine_eres), so their check is effectively off
    "refine_ncheck": 50,
    # inner CG tolerance (r.r < cg_rtol r0.r0) of the FP32 stage and of the
    # refinement of "mixed"; the reference's TN uses 0.1
    "fp32_cg_rtol": 0.1,
    "refine_cg_rtol": 0.01,
    # preconditioned inner CG in the stages of "mixed" (uniform-gas Hessian)
    "mixed_precond": True,
    # preconditioned inner CG for precision "fp64" / "fp32" too (off: the
    # reference's plain CG); for attributing the mixed path's speed-up
    "precond": False,
    # CUDA-event timing of the FP32 potential-only evaluations (stats
    # t_eval_timed / n_eval_timed per stage)
    "time_evals": False,
    # curvature constant of the line search in the stages of "mixed" (None:
    # c2, the reference's 0.2).  The refinement starts from the FP32 density
    # with a Newton step whose length is already right to a few percent; the
    # strong-Wolfe test at 0.2 rejects such steps on the derivative alone and
    # costs two extra FP64 evaluations, so it is relaxed there (at 128^3 Al256
    # the refined energy moves by 1e-9 eV/atom, forces by 1e-6 Ha/bohr)
    "fp32_c2": None,
    "refine_c2": 0.9,
    # FP64 evaluations of the refinement as delta evaluations against its
    # first (full FP64) one: FP32 transforms of the density change, FP64
    # pointwise terms; a full evaluation rebases when the density has moved
    # by more than delta_rtol (relative 2-norm) from the reference
    "refine_delta": True,
    "delta_rtol": 1e-3,
}


class Optimization:
    def __init__(self, optimization_method="CG-HS", optimization_options=None, EnergyEvaluator=None,
                 guess_rho=None):
        self.rho = guess_rho
        self.optimization_options = dict(optimization_options or {})
        for k, v in DEFAULTS.items():
            self.optimization_options.setdefault(k, v)
        if EnergyEvaluator is None:
            raise AttributeError("Must provide an energy evaluator")
        self.EnergyEvaluator = EnergyEvaluator
        self.optimization_method = optimization_method
        self.converged = None
        self.mu = None
        self.energy = None
        self.history = []
        self.stats = {}
        self._functional = None

    # ------------------------------------------------------------------------
    def _check(self):
        if self.optimization_method not in FIRST_ORDER and self.optimization_method != "TN":
            raise AttributeError("The %s direction method not implemented." % self.optimization_method)
        o = self.optimization_options
        if o["algorithm"] != "EMM" or o["vector"] != "Orthogonalization":
            raise NotImplementedError("only algorithm='EMM' with vector='Orthogonalization' is implemented")
        ev = self.EnergyEvaluator
        if self.optimization_method == "TN" and not (isinstance(ev, TotalFunctional) and ev.fusable()):
            raise NotImplementedError("the device optimiser needs a TotalFunctional of this package's "
                                      "functionals (KEDF, XC, HARTREE, PSEUDO)")

    def _run(self, rho, econv, eps, maxiter, maxls=None, hess_rho=None, pred_stop=0.0, eres=0.0, ncheck=None,
             cg_rtol=0.1, pred_next=False, precond=False, c2=None, delta=False, res0_max=0.0):
        o = self.optimization_options
        grid = rho.grid
        plan = grid.plan(rho.dtype)
        L = _lib.load()
        opts = _lib.TnOptions()
        _lib.check(L.gbofdft_tn_options_default(ctypes.byref(opts)))
        opts.econv = float(econv)
        opts.maxfun = int(o["maxfun"])
        opts.maxiter = int(maxiter)
        opts.maxls = int(o["maxls"] if maxls is None else maxls)
        opts.res0_max = float(res0_max or 0.0)
        opts.c1, opts.c2, opts.xtol = float(o["c1"]), float(o["c2"] if c2 is None else c2), float(o["xtol"])
        opts.ncheck = int(o["ncheck"] if ncheck is None else ncheck)
        opts.eps = float(eps)
        opts.pred_stop = float(pred_stop)
        opts.eres = float(eres)
        opts.cg_rtol = float(cg_rtol)
        opts.pred_next = int(bool(pred_next))
        opts.precond = int(bool(precond))
        opts.time_evals = int(bool(o.get("time_evals", False)))
        spec = self.EnergyEvaluator.spec(rho)
        f = spec.ctypes()
        nb = ctypes.c_int64()
        _lib.check(L.gbofdft_tn_workspace_bytes(plan.handle, ctypes.byref(nb)))
        ws = _workspace(grid, rho.dtype, int(nb.value))
        r = rho.as_subclass(torch.Tensor).contiguous()
        res = _lib.TnResult()
        hist = (ctypes.c_double * 4096)()
        res.history = hist
        res.history_cap = 4096
        # torch.ops.gbofdft.optimize_tn(_split): the registered operators over
        # gbofdft_optimize_tn(_split); they return the optimised density
        if hess_rho is None:
            r = torch.ops.gbofdft.optimize_tn(r, torch_ops.handle(plan), ctypes.addressof(f), ctypes.addressof(opts),
                                              ws, int(nb.value), ctypes.addressof(res))
        else:
            hplan = grid.plan(hess_rho.dtype)
            hf = self.EnergyEvaluator.spec(hess_rho).ctypes()
            hb = ctypes.c_int64()
            _lib.check(L.gbofdft_tn_hess_workspace_bytes(hplan.handle, ctypes.byref(hb)))
            hws = _workspace(grid, ("hess", hess_rho.dtype), int(hb.value))
            dstate = grid.delta_state() if delta else None
            if dstate is not None:
                opts.delta = dstate.handle
                opts.delta_rtol = float(o["delta_rtol"])
            r = torch.ops.gbofdft.optimize_tn_split(r, torch_ops.handle(plan), ctypes.addressof(f),
                                                    torch_ops.handle(hplan), ctypes.addressof(hf),
                                                    ctypes.addressof(opts), ws, int(nb.value), hws, int(hb.value),
                                                    ctypes.addressof(res))
        out = dict(energy=res.energy, mu=res.mu, converged=res.converged, n_iter=res.n_iter,
                   n_eval_ev=res.n_eval_ev, n_eval_v=res.n_eval_v, n_eval_hess=res.n_eval_hess,
                   energies=list(res.energies), history=[hist[i] for i in range(res.n_history)],
                   n_sync=res.n_sync, t_sync=res.t_sync, t_total=res.t_total,
                   t_eval_timed=res.t_eval_timed, n_eval_timed=res.n_eval_timed, n_eval_delta=res.n_eval_delta)
        return DirectField(grid, data=r), out

    def optimize_rho(self, guess_rho=None, guess_phi=None, lphi=False):
        """``optimization.py:281-520``: the device TN driver, or the first-order
        methods (``_optimize_first_order``)."""
        if guess_rho is None and self.rho is None:
            raise AttributeError("Must provide a guess density")
        if guess_rho is not None:
            self.rho = guess_rho
        if guess_phi is not None or lphi:
            raise NotImplementedError("guess_phi / lphi are not part of this path")
        self._check()
        o = self.optimization_options
        rho = self.rho
        if not isinstance(rho, DirectField):
            raise TypeError("guess_rho must be a DirectField")
        if self.optimization_method in FIRST_ORDER:
            return self._optimize_first_order(rho)
        prec = o["precision"] or ("fp64" if rho.dtype == torch.float64 else "fp32")
        self.stats = {"stages": []}
        t_start = time.perf_counter()
        if prec in ("fp64", "fp32"):
            dt = torch.float64 if prec == "fp64" else torch.float32
            eps = o["eps"] if o["eps"] is not None else (1e-9 if dt == torch.float64 else o["fp32_eps"])
            r, out = self._run(rho.to(dt) if rho.dtype != dt else rho, o["econv"], eps, o["maxiter"],
                               precond=bool(o["precond"]), res0_max=o["start_residual_max"])
            self.stats["stages"].append(dict(precision=prec, **out))
        elif prec == "mixed":
            # FP32 until its energy changes by less than fp32_econv (default:
            # the 1e-5 eV/atom accuracy gate, 3.67e-7 Ha/atom) or its line
            # search stops resolving progress
            nat = self._natoms()
            e32 = o["fp32_econv"] if o["fp32_econv"] is not None else max(o["econv"], 3.67e-7 * nat)
            r32, out32 = self._run(rho.to(torch.float32), e32, o["fp32_eps"], o["maxiter"],
                                   pred_stop=0.1 * e32, eres=o["fp32_eres"], ncheck=o["stage_ncheck"],
                                   cg_rtol=o["fp32_cg_rtol"], precond=o["mixed_precond"], c2=o["fp32_c2"],
                                   res0_max=o["start_residual_max"])
            self.stats["stages"].append(dict(precision="fp32", **out32))
            if out32["converged"] == 3:
                # the start was rejected (start_residual_max): no refinement
                return self._finish(t_start, rho, out32)
            eps = o["eps"] if o["eps"] is not None else 1e-9
            # the FP32 stage conserves the electron number only to single
            # precision: restore the guess's integral before refining in FP64
            r64 = r32.to(torch.float64)
            n_in = float(rho.as_subclass(torch.Tensor).to(torch.float64).sum())
            n_out = float(r64.as_subclass(torch.Tensor).sum())
            r64 = r64 * (n_in / n_out)
            if o["refine"] not in ("split", "fp64"):
                raise ValueError("refine must be 'split' or 'fp64', got %r" % (o["refine"],))

            def refine(r_start, r_hess):
                if o["refine"] == "split":
                    ps = o["refine_pred_stop"] if o["refine_pred_stop"] is not None else 0.01 * o["econv"]
                    return self._run(r_start, o["econv"], o["fp32_eps"], o["maxiter"], maxls=o["refine_maxls"],
                                     hess_rho=r_hess, pred_stop=ps, eres=o["refine_eres"],
                                     ncheck=o["refine_ncheck"], cg_rtol=o["refine_cg_rtol"], pred_next=True,
                                     precond=o["mixed_precond"], c2=o["refine_c2"], delta=o["refine_delta"])
                return self._run(r_start, o["econv"], eps, o["maxiter"], maxls=o["refine_maxls"],
                                 eres=o["refine_eres"])

            r, out = refine(r64, r32)
            self.stats["stages"].append(dict(precision="fp64", **out))
            # refine_restarts: a refinement whose line search failed while it
            # was still lowering the energy by more than econv starts again
            # from where it stopped
            for _ in range(int(o["refine_restarts"])):
                h = out["history"]
                if not (out["converged"] == 1 and len(h) >= 2 and abs(h[-1] - h[0]) > o["econv"]):
                    break
                r, out = refine(r, r.to(torch.float32))
                self.stats["stages"].append(dict(precision="fp64", restart=True, **out))
            # a refinement whose line search stops on FP64 rounding (no energy
            # change above econv along the last direction) sits at the FP64
            # minimum: report it converged
            h = out["history"]
            if out["converged"] == 1 and len(h) >= 1 and abs(h[-1] - h[0]) <= max(o["econv"], 1e-12 * abs(h[0])) \
                    and out["n_iter"] <= 2:
                out = dict(out, converged=0)
        else:
            raise ValueError("precision must be 'fp64', 'fp32' or 'mixed', got %r" % (prec,))
        if out["converged"] == 3:
            return self._finish(t_start, rho, out)
        return self._finish(t_start, r, out)

    def _finish(self, t_start, r, out):
        self.stats["t_wall"] = time.perf_counter() - t_start
        self.stats["t_glue"] = self.stats["t_wall"] - sum(st["t_total"] for st in self.stats["stages"])
        self.converged = out["converged"]
        self.mu = out["mu"]
        self.energy = out["energy"]
        self.history = out["history"]
        self.rho = r
        self._functional = None
        return r

    # ------------------------------------------------------------------------
    def _optimize_first_order(self, rho):
        """``optimize_rho`` (``optimization.py:281-520``) with a first-order
        direction: the conjugate gradients of ``get_direction_CG``
        (``math_utils.py:396-426``: CG-HS, the reference's default, and CG-PR,
        CG-DY, CG-CD, CG-LS, CG-FR), ``LBFGS`` (``math_utils.py:374-395,
        433-455``; ``h0`` in the options, as the reference requires) or ``GD``.
        The loop is the reference's -- orthogonal rotation of phi, the
        Moré-Thuente line search (the library's ``gbofdft_dcsrch``) on the
        rotation angle, energy-change convergence test -- driven from the host
        with every field on the device: each trial is one evaluation through
        ``torch.ops.gbofdft.eval``, the field algebra and the FP64 reductions
        are device operations on the density's tensors."""
        o = self.optimization_options
        method = self.optimization_method
        grid = rho.grid
        dV = grid.dV
        ev = self.EnergyEvaluator
        t_start = time.perf_counter()
        r = rho.as_subclass(torch.Tensor).to(torch.float64)

        def integral(x):
            return float(x.sum()) * dV

        def evaluate(phi):
            out = ev(DirectField(grid, data=phi * phi), calcType={"E", "V"})
            return float(out.energy), out.potential.as_subclass(torch.Tensor)

        phi = torch.where(r > 0, torch.sqrt(torch.clamp(r, min=0.0)), torch.full_like(r, 1e-300))
        phi = phi * np.sqrt(float(r.sum()) / float((phi * phi).sum()))
        energy, pot = evaluate(phi)
        n_eval = 1

        def mu_of(pot, phi):
            rr = phi * phi
            return integral(pot * rr) / integral(rr)

        mu = mu_of(pot, phi)
        res_a = [(pot - mu) * phi]
        dir_a = []
        history = [energy]
        lbfgs = _Lbfgs(o["h0"], o["maxcor"]) if method == "LBFGS" else None
        theta = 0.1
        converged = 1
        L = _lib.load()
        it = 0
        for it in range(1, o["maxiter"]):
            p = _direction(method, res_a, dir_a, lbfgs)
            p, theta0 = _orthonormalize(p, phi, dV)
            if 2.0 * float((pot * phi * p).sum()) > 0:
                p, theta0 = _orthonormalize(-res_a[-1], phi, dV)   # "Change to steepest descent"
            theta = min(theta0, theta)

            def value_deriv(t, phi=phi, p=p):
                newphi = phi * np.cos(t) + p * np.sin(t)
                e, v = evaluate(newphi)
                p2 = p * np.cos(t) - phi * np.sin(t)
                return e, 2.0 * float((v * newphi * p2).sum()) * dV, (newphi, e, v)

            g0 = 2.0 * float((pot * phi * p).sum()) * dV
            theta, payload, nls = _line_search(L, value_deriv, theta, energy, g0, o["c1"], o["c2"], np.pi, 0.0,
                                               o["xtol"], o["maxls"])
            n_eval += nls
            if theta is None:
                converged = 1
                break
            old_phi = phi
            phi, energy, pot = payload
            mu = mu_of(pot, phi)
            res_a.append((pot - mu) * phi)
            if lbfgs is not None:
                lbfgs.update(phi - old_phi, res_a[-1] - res_a[-2])
            history.append(energy)
            if len(history) - 1 >= o["ncheck"] and all(abs(history[-2 - i] - energy) <= o["econv"]
                                                          for i in range(o["ncheck"])):
                converged = 0
                break
            dir_a.append(p)
            if len(res_a) > 2:
                res_a.pop(0)
            if len(dir_a) > 2:
                dir_a.pop(0)
        else:
            converged = 2
        out_rho = DirectField(grid, data=(phi * phi).to(rho.dtype))
        self.stats = {"stages": [dict(precision="fp64" if rho.dtype == torch.float64 else "fp32", method=method,
                                      energy=energy, mu=mu, converged=converged, n_iter=it, n_eval_ev=n_eval,
                                      n_eval_v=0, n_eval_hess=0, energies=[], history=list(history), n_sync=0,
                                      t_sync=0.0, t_total=time.perf_counter() - t_start)],
                      "t_wall": time.perf_counter() - t_start, "t_glue": 0.0}
        self.converged = converged
        self.mu = mu
        self.energy = energy
        self.history = history
        self.rho = out_rho
        self._functional = None
        return out_rho

    def optimize_rho_multistep(self, guess_rho, multistep=2, nr_final=None):
        """Coarse-to-fine optimisation (the multi-step branch of
        ``OptimizeDensityConf``, ``interface.py:160-200``): optimise on the
        guess's grid, then ``multistep - 1`` times double the grid (the last
        step goes to ``nr_final`` when given), interpolate the density's
        spectrum onto it (``field2distrib``), rescale it to the electron
        count, move the local pseudopotential to the new grid and optimise
        again.  Returns the density on the finest grid."""
        from .grid import DirectGrid
        from .utils import field2distrib
        if multistep < 1:
            raise ValueError("multistep must be >= 1")
        charge_total = float(np.sum(guess_rho.integral()))
        rho = self.optimize_rho(guess_rho=guess_rho)
        nr = np.array(guess_rho.grid.nrR, dtype=int)
        for istep in range(2, multistep + 1):
            if istep == multistep and nr_final is not None:
                nr = np.array(nr_final, dtype=int)
            else:
                nr = nr * 2
            grid2 = DirectGrid(lattice=rho.grid.lattice, nr=nr, full=rho.grid.full)
            rho_ini = DirectField(grid2, rank=rho.rank, dtype=rho.dtype)
            field2distrib(rho, rho_ini, root=0)
            rho_ini = rho_ini * (charge_total / float(np.sum(rho_ini.integral())))
            for f in self.EnergyEvaluator.funcDict.values():
                if getattr(f, "type", None) == "PSEUDO":
                    f.restart(full=False, ions=f.ions, grid=grid2)
            rho = self.optimize_rho(guess_rho=rho_ini)
        return rho

    def _natoms(self):
        for f in self.EnergyEvaluator.funcDict.values():
            if getattr(f, "type", None) == "PSEUDO":
                return f.ions.nat
        return 1

    @property
    def functional(self):
        if self._functional is None and self.rho is not None:
            self._functional = self.EnergyEvaluator(self.rho, calcType={"E", "V"})
        return self._functional

    def __call__(self, guess_rho=None, calcType={"E", "V"}, guess_phi=None, lphi=False):
        return self.optimize_rho(guess_rho=guess_rho, guess_phi=guess_phi, lphi=lphi)


FIRST_ORDER = ("CG-HS", "CG", "CG-PR", "CG-DY", "CG-CD", "CG-LS", "CG-FR", "LBFGS", "GD")


def _dot(a, b):
    return float((a * b).sum())


def _direction(method, res_a, dir_a, lbfgs):
    """``get_direction`` of the first-order methods (``math_utils.py:396-455``)."""
    r1 = res_a[-1]
    if method == "GD":
        return -r1
    if method == "LBFGS":
        q = -r1
        alphas = [0.0] * len(lbfgs.s)
        # the reference's loop stops before i = 0
        for i in range(len(lbfgs.s) - 1, 0, -1):
            a = lbfgs.rho[i] * _dot(lbfgs.s[i], q)
            alphas[i] = a
            q = q - a * lbfgs.y[i]
        if not lbfgs.H0:
            gamma = 1.0 if len(lbfgs.s) < 1 else _dot(lbfgs.s[-1], lbfgs.y[-1]) / _dot(lbfgs.y[-1], lbfgs.y[-1])
            d = gamma * q
        else:
            d = lbfgs.H0 * q
        for i in range(len(lbfgs.s)):
            b = lbfgs.rho[i] * _dot(lbfgs.y[i], d)
            d = d + lbfgs.s[i] * (alphas[i] - b)
        return d
    if len(res_a) == 1:
        beta = 0.0
    else:
        r0 = res_a[-2]
        d0 = dir_a[-1] if dir_a else None
        if method in ("CG-HS", "CG") and d0 is not None:
            dr = r1 - r0
            beta = _dot(r1, dr) / _dot(d0, dr)
        elif method == "CG-PR":
            beta = max(_dot(r1, r1 - r0) / _dot(r0, r0), 0.0)
        elif method == "CG-DY" and d0 is not None:
            beta = _dot(r1, r1) / _dot(d0, r1 - r0)
        elif method == "CG-CD" and d0 is not None:
            # kept as the reference has it: -(r1 ** 2) / sum(d0 r0) is a field,
            # so the update is pointwise
            beta = -(r1 * r1) / _dot(d0, r0)
        elif method == "CG-LS" and d0 is not None:
            beta = _dot(r1, r1 - r0) / _dot(d0, r0)
        else:
            beta = _dot(r1, r1) / _dot(r0, r0)
    if not dir_a:
        return -r1
    return -r1 + beta * dir_a[-1]


def _orthonormalize(p, phi, dV):
    """``OrthogonalNormalization`` (``optimization.py:204-225``), vector
    "Orthogonalization"."""
    ne = float((phi * phi).sum()) * dV
    p = p - (float((p * phi).sum()) * dV / ne) * phi
    pn = float((p * p).sum()) * dV
    return p * np.sqrt(ne / pn), float(np.sqrt(pn / ne))


class _Lbfgs:
    """``LBFGS`` history (``math_utils.py:374-395``): at most Bound + 1 pairs."""

    def __init__(self, H0=1.0, Bound=5):
        self.H0, self.Bound = H0, Bound
        self.s, self.y, self.rho = [], [], []

    def update(self, dx, dg):
        if len(self.s) > self.Bound:
            self.s.pop(0)
            self.y.pop(0)
            self.rho.pop(0)
        self.s.append(dx)
        self.y.append(dg)
        self.rho.append(1.0 / _dot(dg, dx))


def _line_search(L, func, alpha0, f0, g0, c1, c2, amax, amin, xtol, maxiter):
    """``LineSearchDcsrch2`` (``math_utils.py:76-106``) with the library's
    More-Thuente state machine; returns (alpha or None, payload, trials)."""
    state = (ctypes.c_double * 32)()
    state[0], state[1], state[2], state[3], state[4] = c1, c2, xtol, amin, amax
    stp = ctypes.c_double(alpha0)
    f, g = f0, g0
    task = 0
    payload = None
    trials = 0
    for _ in range(maxiter):
        task = L.gbofdft_dcsrch(state, 32, ctypes.byref(stp), float(f), float(g), task)
        if task < 0:
            raise RuntimeError("gbofdft_dcsrch: %s" % _lib.last_error())
        if task == 1:
            f, g, payload = func(stp.value)
            trials += 1
        else:
            break
    else:
        return None, payload, trials
    if task in (3, 4):
        return None, payload, trials
    return stp.value, payload, trials


def _workspace(grid, dtype, nbytes):
    """Per-(grid, dtype) device workspace for the optimiser, kept with the
    grid's plans (allocated once, freed with the grid)."""
    key = ("tn_workspace", dtype)
    t = grid._plans.get(key)
    if t is None or t.numel() * 8 < nbytes + 512:
        t = torch.empty(nbytes // 8 + 64, dtype=torch.float64, device="cuda")
        grid._plans[key] = t
    return t
