"""Physical constants in ASE's unit system (eV, Angstrom), CODATA 2014.

Golden-fixture shim only: the reference imports ``ase.units`` for unit
conversions (``dftpy/constants.py:3``).  The values follow from the CODATA
2014 fundamental constants; none of them enters the OF-DFT arithmetic in
atomic units, they only convert printouts.
"""
import math

_c = 299792458.0                 # speed of light, m/s
_mu0 = 4.0e-7 * math.pi          # vacuum permeability
_eps0 = 1.0 / _mu0 / _c ** 2     # vacuum permittivity (evaluated in ase's order)
_hplanck = 6.626070040e-34       # Planck constant, J s
_hbar = _hplanck / (2.0 * math.pi)
_e = 1.6021766208e-19            # elementary charge, C
_me = 9.10938356e-31             # electron mass, kg
_amu = 1.660539040e-27           # atomic mass unit, kg
_k = 1.38064852e-23              # Boltzmann constant, J/K
_Nav = 6.022140857e23

Ang = Angstrom = 1.0
nm = 10.0
m = 1.0e10
eV = 1.0
J = 1.0 / _e
kJ = 1000.0 * J
C = 1.0 / _e
s = 1.0e10 * math.sqrt(_e / _amu)
second = s
fs = 1.0e-15 * s
kg = 1.0 / _amu
Pascal = (1.0 / _e) / 1.0e30
GPa = 1.0e9 * Pascal
bar = 1.0e5 * Pascal
alpha = _e * _e / (4.0 * math.pi * _eps0) / _hbar / _c
Bohr = 4.0e10 * math.pi * _eps0 * _hbar ** 2 / _me / _e ** 2
Hartree = Ha = _me * _e ** 3 / 16.0 / math.pi ** 2 / _eps0 ** 2 / _hbar ** 2
Rydberg = Ry = 0.5 * Hartree
AUT = _hbar / (Hartree * _e) * s
kB = _k / _e
