"""Functionals with the reference's ``dftpy.functional`` interface
(``functional/__init__.py:20-50``)."""
from .kedf import KEDF
from .output import AbstractFunctional, FunctionalOutput, ZeroFunctional
from .pseudo import AnalyticPP, LocalPseudo, ewald
from .total_functional import TotalFunctional
from .xc_hartree import XC, Hartree

FunctionalTypeDict = {"KEDF": KEDF, "PSEUDO": LocalPseudo, "HARTREE": Hartree, "XC": XC}


def Functional(type=None, optional_kwargs=None, **kwargs):
    """Factory: ``Functional(type='KEDF', name='WT')`` etc."""
    type = type.upper()
    if optional_kwargs is not None:
        kwargs.update(optional_kwargs)
    try:
        cls = FunctionalTypeDict[type]
    except KeyError:
        raise AttributeError("Unknown functional type: {}.".format(type))
    return cls(**kwargs)


__all__ = ["Functional", "FunctionalOutput", "AbstractFunctional", "ZeroFunctional", "TotalFunctional", "KEDF",
           "XC", "Hartree", "LocalPseudo", "AnalyticPP", "ewald"]
