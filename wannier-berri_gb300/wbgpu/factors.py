"""Physical prefactors (same definitions as the reference factors.py:1-36, from scipy.constants)."""
from scipy.constants import elementary_charge, hbar, physical_constants, angstrom

bohr = physical_constants['Bohr radius'][0] / angstrom
eV_au = physical_constants['electron volt-hartree relationship'][0]
factor_ahc = -(elementary_charge ** 2 / hbar / angstrom)
factor_opt = -factor_ahc
factor_morb = -eV_au / bohr ** 2
