"""Physical prefactors (same definitions as the reference factors.py:1-36, from scipy.constants)."""
from scipy.constants import elementary_charge, hbar, physical_constants, angstrom, pi, electron_mass

bohr = physical_constants['Bohr radius'][0] / angstrom
eV_au = physical_constants['electron volt-hartree relationship'][0]
factor_ahc = -(elementary_charge ** 2 / hbar / angstrom)
factor_opt = -factor_ahc
factor_morb = -eV_au / bohr ** 2
TAU_UNIT = 1e-15  # relaxation time unit, fs (factors.py:3)
factor_ohmic = (elementary_charge ** 2 / hbar / angstrom * TAU_UNIT * elementary_charge / hbar)  # factors.py:26
factor_shc = -factor_ahc  # factors.py:37
# factors.py:50-51
factor_shift_current = hbar / elementary_charge * pi * elementary_charge ** 3 / (4 * hbar ** 2)
factor_injection_current = - pi * elementary_charge ** 3 / (hbar ** 2) * TAU_UNIT
factor_nlahc = elementary_charge ** 3 / hbar ** 2 * TAU_UNIT  # factors.py:28
factor_nldrude = -(elementary_charge ** 3 / hbar ** 2 * TAU_UNIT ** 2 * elementary_charge / hbar)  # factors.py:31-32
factor_hall_classic = -(elementary_charge ** 3 / hbar ** 2 * angstrom * TAU_UNIT ** 2 *
                        elementary_charge ** 2 / hbar ** 2)  # factors.py:29-30, with tau^2 E^1 B^1
bohr_magneton = elementary_charge * hbar / (2 * electron_mass)  # factors.py:6
fac_orb_Z = elementary_charge / 2 / hbar * angstrom ** 2  # factors.py:16: m_orb B in eV
fac_spin_Z = hbar / (2 * electron_mass)  # factors.py:17: m_spin B in eV
factor_gme_spin = -bohr_magneton / angstrom ** 2  # factors.py:22
factor_gme_orb = -(elementary_charge * angstrom ** 2) * elementary_charge / (2 * hbar) / angstrom ** 2  # factors.py:12,20
