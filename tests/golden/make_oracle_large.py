"""Oracle evaluation of the 4000-atom LMGP workload at its full size (360^3).

Run from the repository root: ``python tests/golden/make_oracle_large.py``
(about 10 GB of memory and a few minutes on one core).

The reference's LMGP (``kedf/lwt.py:82-341``) is restated by the numpy oracle
(``oracle/ofdft.py`` ``LWTNL``), which is pinned to the reference's own LMGP
test values on its test density; running the reference itself at 360^3 is not
needed for the fixture.  Structure: ``systems.config_al4000(0)`` (10x10x10 fcc
Al, jitter 0.1 Bohr).  Density: the superposed Gaussian atomic densities of
``get_3d_value_recipe`` (PME, ``density/density.py:252-300``), a fixed density
the GPU reproduces to round-off.  Functional: TF + vW + LMGP (linear, kdd 3)
+ LDA + Hartree + analytic local PP (PME) + Ewald.

al4000_oracle.npz holds the energy of every term, the number of k_F knots,
the total and nonlocal potentials at 4096 fixed random grid points (and the
density there, to check both sides used the same one), checksums of the
total potential, and the PP and Ewald forces on all 4000 atoms.
"""
import os
import pathlib
import sys
import time

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
ROOT = HERE.parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

NSAMPLE = 4096


def main():
    from dftpy_gb300 import systems
    from oracle import ofdft as O
    t0 = time.perf_counter()
    st = systems.config_al4000(0)
    ev = O.OFDFT(st.lattice, st.nr, st.positions, st.symbols, kedf="TFVW")
    g = ev.grid
    tab = {"Al": systems.atomic_density_table(3.0, systems.ATOMIC_SIGMA["Al"])}
    rho = O.density_guess_recipe(g, st.positions, st.symbols, tab, st.nelec, pme=True)
    t1 = time.perf_counter()
    comps = ev.components(rho)
    lw = O.LWTNL("MGP", "linear")
    e_nl, v_nl = lw(rho, g, calc_e=True, calc_v=True)
    pot = v_nl.copy()
    for k in comps:
        pot += comps[k][1]
    t2 = time.perf_counter()
    f_pp = O.pp_forces_pme(rho, g, st.positions, st.symbols, ev.tables)
    f_ii = O.ewald_forces(g, st.positions, ev.charges, pme=True)
    t3 = time.perf_counter()
    idx = np.sort(np.random.default_rng(0).choice(rho.size, NSAMPLE, replace=False))
    energies = {k: float(comps[k][0]) for k in comps}
    energies["NL"] = float(e_nl)
    energies["II"] = float(ev.ewald["energy"])
    out = {"E_" + k: v for k, v in energies.items()}
    out["E_total"] = sum(energies.values())
    np.savez(HERE / "al4000_oracle.npz", nr=np.array(st.nr), nat=st.nat, nknots=int(lw.last_knots.size),
             sample_idx=idx, rho_s=rho.ravel()[idx], V_s=pot.ravel()[idx], Vnl_s=v_nl.ravel()[idx],
             V_sum=float(pot.sum()), V_absmax=float(np.abs(pot).max()), V_rho=float((pot * rho).sum() * g.dV),
             forces_pp=f_pp, forces_ii=f_ii, t_density=t1 - t0, t_eval=t2 - t1, t_forces=t3 - t2, **out)
    print("wrote", HERE / "al4000_oracle.npz", {k: round(v, 8) for k, v in out.items()},
          "knots", int(lw.last_knots.size), "times %.0f %.0f %.0f s" % (t1 - t0, t2 - t1, t3 - t2))


if __name__ == "__main__":
    main()
