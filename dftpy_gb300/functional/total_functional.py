"""Sum of functionals (``functional/total_functional.py``).

When every member is one of this package's functionals (KEDF, XC, HARTREE,
PSEUDO), ``compute`` issues ONE fused device evaluation (``gbofdft_eval``):
one read of rho, shared transform passes, one write of the total potential.
Any other AbstractFunctional falls back to summing the members' outputs.
"""
import numpy as np

from .. import _lib
from .kedf import KEDF
from .output import AbstractFunctional, FunctionalOutput
from .pseudo import LocalPseudo
from .xc_hartree import XC, Hartree
from ._eval import Spec, evaluate

_FUSABLE = (KEDF, XC, Hartree, LocalPseudo)


class TotalFunctional(AbstractFunctional):
    def __init__(self, ewald=None, **kwargs):
        self.funcDict = {k: v for k, v in kwargs.items() if v is not None}
        self.UpdateNameType()
        self._ewald = ewald

    def __repr__(self):
        return self.funcDict.__repr__()

    def __getitem__(self, key):
        return self.funcDict[key]

    def __setitem__(self, key, value):
        self.funcDict.update({key: value})
        self.UpdateNameType()

    def UpdateNameType(self):
        """``total_functional.py:67-76``: members must be AbstractFunctional."""
        self.name = ""
        self.type = ""
        for key, f in self.funcDict.items():
            if not isinstance(f, AbstractFunctional):
                raise TypeError("{} must be AbstractFunctional".format(key))
            setattr(self, key, f)
            self.name += getattr(f, "name") + " "
            self.type += getattr(f, "type") + " "

    def UpdateFunctional(self, keysToRemove=[], newFuncDict={}):
        for key in keysToRemove:
            self.funcDict.pop(key, None)
        self.funcDict.update(newFuncDict)
        self.UpdateNameType()

    def Subset(self, keys):
        return TotalFunctional(**{k: self.funcDict[k] for k in keys})

    @property
    def ewald(self):
        if self._ewald is not None:
            return self._ewald
        for f in self.funcDict.values():
            if getattr(f, "type", None) == "PSEUDO":
                return f.get_ewald()
        return None

    def fusable(self):
        return all(isinstance(f, _FUSABLE) for f in self.funcDict.values())

    def spec(self, rho):
        """Merged component description of all members (fused path)."""
        sp = Spec()
        for f in self.funcDict.values():
            sp = sp.merge(f.spec(rho))
        ew = self.ewald
        sp.e_ion = float(ew.energy) if ew is not None else 0.0
        return sp

    def compute(self, rho, calcType={"E", "V"}, **kwargs):
        return self.get_energy_potential(rho, calcType=calcType, **kwargs)

    def Energy(self, rho, **kwargs):
        return self.compute(rho, calcType={"E"}).energy

    def get_energy_potential(self, rho, calcType={"E", "V"}, split=False, **kwargs):
        if self.fusable() and not split:
            en, pot = evaluate(rho, self.spec(rho), set(calcType) | {"V"})
            out = FunctionalOutput(name="TOTAL", energy=0.0 if en is None else float(en[_lib.E_TOTAL]))
            if "V" in calcType:
                out.potential = pot
            if en is not None:
                self.last_energies = en
            return out
        parts = {"TOTAL": FunctionalOutput(name="TOTAL", energy=0.0)}
        for key, func in self.funcDict.items():
            res = func(rho, calcType=calcType, **kwargs)
            if split:
                parts[getattr(func, "type", key)] = res
            parts["TOTAL"] = parts["TOTAL"] + res
        ew = self.ewald
        if ew is not None:
            r = FunctionalOutput(name="II", energy=ew.energy)
            if split:
                parts["II"] = r
            parts["TOTAL"] = parts["TOTAL"] + r
        return parts if split else parts["TOTAL"]

    def get_forces(self, rho, ions=None, split=False, **kwargs):
        """Forces on the ions, nat x 3 (Ha/Bohr) (``get_forces``,
        ``total_functional.py:148-174``): every member with a ``forces`` method
        plus the Ewald forces; ``split=True`` returns them by member key with
        the Ewald part under ``"II"`` and the sum under ``"TOTAL"``."""
        ew = self.ewald
        if ions is None:
            if ew is None:
                raise ValueError("Please provide ions for forces")
            ions = ew.ions
        forces = {"TOTAL": np.zeros((ions.nat, 3))}
        for key, func in self.funcDict.items():
            if hasattr(func, "forces"):
                f = func.forces(rho)
                if f is not None:
                    if split:
                        forces[key] = f
                    forces["TOTAL"] = forces["TOTAL"] + f
        if ew is not None:
            f = ew.forces
            if split:
                forces["II"] = f
            forces["TOTAL"] = forces["TOTAL"] + f
        return forces if split else forces["TOTAL"]

    def get_stress(self, rho, split=False, **kwargs):
        """Stress tensor, 3x3 (Ha/Bohr^3) (``get_stress``, ``total_functional.py:176-209``):
        the KEDF parts under "KEDF-TF", "KEDF-VW", "KEDF-NL", then "XC",
        "HARTREE", "PSEUDO", the Ewald part under "II" and the sum under
        "TOTAL" with ``split=True``.  The density terms come from one energy
        evaluation and one ``gbofdft_stress_functional`` call."""
        from .stress import functional_stress
        stress = {"TOTAL": np.zeros((3, 3))}
        own = [f for f in self.funcDict.values() if isinstance(f, _FUSABLE)]
        if own:
            sp = Spec()
            for f in own:
                sp = sp.merge(f.spec(rho))
            en, _ = evaluate(rho, sp, {"E"})
            parts = functional_stress(rho, sp, en)
            for k, v in parts.items():
                stress[("KEDF-" + k) if k in ("TF", "VW", "NL") else k] = v
            for f in own:
                if isinstance(f, LocalPseudo):
                    stress["PSEUDO"] = f.stress(rho, energy=float(en[_lib.E_PSEUDO]))
        for key, f in self.funcDict.items():
            if not isinstance(f, _FUSABLE):
                stress[getattr(f, "type", key)] = f.stress(rho)
        ew = self.ewald
        if ew is not None:
            stress["II"] = ew.stress
        stress["TOTAL"] = sum(v for k, v in stress.items() if k != "TOTAL")
        return stress if split else stress["TOTAL"]
