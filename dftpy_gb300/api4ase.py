"""ASE calculator (``api/api4ase.py:11-119`` ``DFTpyCalculator``, evaluator path).

``DFTpyCalculator(evaluator=TotalFunctional(...), rho=initial_density)``
optimises the density for each new atomic configuration, starting from the
previous step's density (the density is reused between ionic steps), and
returns the energy (eV), forces (eV/A) and stress (eV/A^3, Voigt order xx yy
zz yz xz xy) of ASE's unit system.  Positions and cell change through
``LocalPseudo.restart``; a new cell keeps the grid's point counts and rescales
the density to the electron count.  When ``ase`` is importable the class is an
``ase.calculators.calculator.Calculator``; otherwise it offers the same
``get_potential_energy`` / ``get_forces`` / ``get_stress`` calls on any object
with ``positions`` (A), ``cell`` (A) and chemical symbols.
"""
import numpy as np
import torch

from .field import DirectField
from .grid import DirectGrid
from .ions import Ions
from .optimization import Optimization
from .pseudo_files import BOHR_ANG, HARTREE_EV

ENERGY_CONV = HARTREE_EV                   # Ha -> eV
FORCE_CONV = HARTREE_EV / BOHR_ANG         # Ha/Bohr -> eV/A
STRESS_CONV = HARTREE_EV / BOHR_ANG ** 3   # Ha/Bohr^3 -> eV/A^3

try:
    from ase.calculators.calculator import Calculator as _Base, all_changes as _ALL
except Exception:                          # ase is optional
    _Base, _ALL = object, ["positions", "numbers", "cell", "pbc"]


def ions_from_atoms(atoms):
    """``Ions.from_ase``: Angstrom -> Bohr."""
    cell = np.asarray(getattr(atoms.cell, "array", atoms.cell), dtype=float) / BOHR_ANG
    pos = np.asarray(atoms.get_positions() if hasattr(atoms, "get_positions") else atoms.positions,
                     dtype=float) / BOHR_ANG
    sym = atoms.get_chemical_symbols() if hasattr(atoms, "get_chemical_symbols") else list(atoms.symbols)
    return Ions(list(sym), positions=pos, cell=cell)


class DFTpyCalculator(_Base):
    implemented_properties = ["energy", "forces", "stress"]

    def __init__(self, config=None, mp=None, optimizer=None, evaluator=None, rho=None, zero_stress=False,
                 **kwargs):
        if config is not None:
            raise NotImplementedError("the config-file driver is not part of this path; pass an evaluator")
        if _Base is not object:
            _Base.__init__(self, **kwargs)
        else:
            self.results = {}
            self.atoms = None
        self.optimizer = optimizer
        self.evaluator = evaluator
        self.zero_stress = zero_stress
        self.dftpy_results = {"density": rho}
        self._state = None

    # -- ase-independent state tracking -------------------------------------
    def _changes(self, atoms):
        if self._state is None:
            return list(_ALL)
        pos, cell, sym = self._state
        ch = []
        ions = ions_from_atoms(atoms)
        if not np.array_equal(ions.cell, cell):
            ch.append("cell")
        if not np.array_equal(ions.positions, pos):
            ch.append("positions")
        if list(ions.symbols) != sym:
            ch.append("numbers")
        return ch

    def calculate(self, atoms=None, properties=("energy",), system_changes=_ALL):
        if _Base is not object:
            _Base.calculate(self, atoms, properties, system_changes)
        else:
            if atoms is not None:
                self.atoms = atoms
            system_changes = self._changes(self.atoms)
        if len(system_changes) > 0:
            self.run(system_changes, properties)
        res = self.dftpy_results
        self.results["energy"] = res["energy"] * ENERGY_CONV
        if "forces" in properties:
            if res.get("forces") is None:
                res["forces"] = self.evaluator.get_forces(res["density"])
            self.results["forces"] = res["forces"] * FORCE_CONV
        if "stress" in properties:
            voigt = np.zeros(6)
            if not self.zero_stress:
                if res.get("stress") is None:
                    res["stress"] = self.evaluator.get_stress(res["density"])
                s = res["stress"]
                voigt = np.array([s[0, 0], s[1, 1], s[2, 2], s[1, 2], s[0, 2], s[0, 1]])
            self.results["stress"] = voigt * STRESS_CONV

    def run(self, system_changes=_ALL, properties=("energy",)):
        """``run_normal`` (``api4ase.py:63-98``)."""
        if self.evaluator is None:
            raise ValueError("!!!Error: Please give a 'config' or 'evaluator' for the calculator")
        rho = self.dftpy_results.get("density")
        if rho is None:
            raise ValueError("!!!Error: Please give a initial density for the calculator")
        ions = ions_from_atoms(self.atoms)
        grid = rho.grid
        if "cell" in system_changes:
            # same point counts on the new cell (field2distrib of a serial run)
            grid = DirectGrid(ions.cell, tuple(int(x) for x in grid.nrR), full=grid.full)
            rho = DirectField(grid, data=rho.as_subclass(torch.Tensor).clone())
        for func in self.evaluator.funcDict.values():
            if getattr(func, "type", None) == "PSEUDO":
                func.restart(ions=ions, grid=grid)
        if "cell" in system_changes:
            x = rho.as_subclass(torch.Tensor) * (self._nelec(rho) / rho.integral())
            rho = DirectField(grid, data=x)
        if self.optimizer is None:
            self.optimizer = Optimization(EnergyEvaluator=self.evaluator, optimization_method="TN")
        rho = self.optimizer.optimize_rho(guess_rho=rho)
        self.dftpy_results = {"density": rho, "energy": float(self.evaluator.Energy(rho)), "forces": None,
                              "stress": None}
        self._state = (ions.positions.copy(), ions.cell.copy(), list(ions.symbols))

    def _nelec(self, rho):
        for func in self.evaluator.funcDict.values():
            if getattr(func, "type", None) == "PSEUDO":
                return func.ions.get_ncharges()
        return float(rho.integral())

    # -- the ase Calculator calls, for use without ase -----------------------
    if _Base is object:
        def get_potential_energy(self, atoms=None, force_consistent=False):
            self.calculate(atoms, ["energy"])
            return self.results["energy"]

        def get_forces(self, atoms=None):
            self.calculate(atoms, ["energy", "forces"])
            return self.results["forces"]

        def get_stress(self, atoms=None):
            self.calculate(atoms, ["energy", "stress"])
            return self.results["stress"]
