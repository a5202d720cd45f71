"""Functional base class and output container (``functional/abstract_functional.py``,
``functional/functional_output.py``)."""
import copy
from abc import ABC, abstractmethod


class AbstractFunctional(ABC):
    """Anything with ``compute(rho, calcType) -> FunctionalOutput``
    (``abstract_functional.py:12-30``)."""

    @abstractmethod
    def __init__(self):
        pass

    def __repr__(self):
        return getattr(self, "name", self.__class__.__name__) + ", " + repr(self.__dict__)

    def __call__(self, rho, *args, **kwargs):
        return self.compute(rho, *args, **kwargs)

    @abstractmethod
    def compute(self, rho, *args, **kwargs):
        pass


class FunctionalOutput:
    """Energy (float, Ha) and potential (DirectField) of a functional, with the
    reference's ``+ - * /`` algebra (``functional_output.py:8-112``)."""

    attr_list = ["energy", "potential", "energydensity", "v2rho2", "v3rho3", "v4rho4", "force", "stress"]

    def __init__(self, name=None, energy=None, potential=None, energydensity=None, v2rho2=None, v3rho3=None,
                 v4rho4=None, force=None, stress=None):
        if name is None:
            raise AttributeError("Functional name must be specified")
        self.name = name
        for key, value in (("energy", energy), ("potential", potential), ("energydensity", energydensity),
                           ("v2rho2", v2rho2), ("v3rho3", v3rho3), ("v4rho4", v4rho4), ("force", force),
                           ("stress", stress)):
            if value is not None:
                setattr(self, key, value)

    def __iter__(self):
        for key in self.attr_list:
            if hasattr(self, key):
                yield key, getattr(self, key)

    def sum(self, other=None):
        if other is None:
            return self.copy()
        name = self.name if self.name == other.name else self.name + other.name
        result = FunctionalOutput(name=name)
        for key, value in self:
            setattr(result, key, value + getattr(other, key) if hasattr(other, key) else value)
        for key, value in other:
            if not hasattr(result, key):
                setattr(result, key, value)
        return result

    def sub(self, other):
        result = self.copy()
        for key, value in self:
            setattr(result, key, value - getattr(other, key) if hasattr(other, key) else value)
        for key, value in other:
            if not hasattr(result, key):
                setattr(result, key, -value)
        return result

    def mul(self, x):
        result = self.copy()
        for key, value in result:
            setattr(result, key, value * x)
        return result

    def div(self, x):
        if x == 0:
            raise ValueError("Dividing zero")
        result = self.copy()
        for key, value in result:
            setattr(result, key, value / x)
        return result

    __add__ = sum
    __sub__ = sub
    __mul__ = mul
    __truediv__ = div

    def copy(self):
        out = FunctionalOutput(name=self.name)
        for key, value in self:
            setattr(out, key, value.clone() if hasattr(value, "clone") else copy.deepcopy(value))
        return out


class ZeroFunctional:
    """``functional_output.py:114-131``."""

    def __init__(self, *args, **kwargs):
        pass

    def __call__(self, rho, *args, **kwargs):
        return self.compute(rho, *args, **kwargs)

    @staticmethod
    def compute(rho, *args, calcType={"E", "V"}, **kwargs):
        from ..field import DirectField
        out = FunctionalOutput(name="ZERO", energy=0.0)
        if "V" in calcType:
            out.potential = DirectField(grid=rho.grid, dtype=rho.dtype)
        return out
