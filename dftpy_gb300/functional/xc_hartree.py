"""Exchange-correlation (``functional/xc/__init__.py``) and Hartree
(``functional/hartree.py``) functionals."""
from .. import _lib
from .output import AbstractFunctional, FunctionalOutput
from ._eval import Spec, evaluate


class XC(AbstractFunctional):
    """Perdew-Zunger LDA (``xc/semilocal_xc.py:253-290``); libxc is not part of
    this path."""

    def __init__(self, xc=None, core_density=None, libxc=None, name=None, pseudo=None, **kwargs):
        xc = xc or name
        self.type = "XC"
        self.name = xc or "XC"
        if not xc and not libxc:
            raise ValueError("Please give a 'xc' or 'libxc'.")
        if (xc or "").lower() != "lda" or libxc not in (None, False):
            raise ModuleNotFoundError("only xc='LDA' is available (pylibxc paths are not part of this build)")
        if core_density is not None:
            raise NotImplementedError("non-linear core correction is not part of this path")
        self.options = dict(kwargs)
        self.energy = None

    def spec(self, rho):
        sp = Spec()
        sp.xc = 1
        return sp

    def stress(self, density, **kwargs):
        """``XC.stress`` -> ``LDAStress`` (``xc/__init__.py:83-88``, ``semilocal_xc.py:308-322``)."""
        from .stress import functional_stress
        return functional_stress(density, self.spec(density))["XC"]

    def compute(self, density, calcType={"E", "V"}, **kwargs):
        en, pot = evaluate(density, self.spec(density), calcType)
        out = FunctionalOutput(name="XC")
        if en is not None:
            out.energy = float(en[_lib.E_XC])
            self.energy = out.energy
        if "V" in calcType:
            out.potential = pot
        return out


class Hartree(AbstractFunctional):
    """v_H = ifft(4 pi rho(G) / G^2), E = 1/2 int v_H rho (``hartree.py:24-45``)."""

    def __init__(self, **kwargs):
        self.type = "HARTREE"
        self.name = "HARTREE"
        self.options = kwargs
        self._energy = None

    def __repr__(self):
        return "HARTREE"

    def spec(self, rho):
        sp = Spec()
        sp.hartree = True
        return sp

    def stress(self, density, **kwargs):
        """``Hartree.stress`` (``hartree.py:51-90``)."""
        from .stress import functional_stress
        return functional_stress(density, self.spec(density))["HARTREE"]

    def compute(self, density, calcType={"E", "V"}, **kwargs):
        en, pot = evaluate(density, self.spec(density), calcType)
        out = FunctionalOutput(name="Hartree", energy=0 if en is None else float(en[_lib.E_HARTREE]))
        if "V" in calcType:
            out.potential = pot
        if en is not None:
            self._energy = out.energy
        return out

    @property
    def energy(self):
        return self._energy
