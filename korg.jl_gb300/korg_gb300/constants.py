"""Physical constants in cgs / eV, the values Korg.jl uses (src/constants.jl:3-19)."""

kboltz_cgs = 1.380649e-16  # erg/K
hplanck_cgs = 6.62607015e-27  # erg*s
c_cgs = 2.99792458e10  # cm/s
electron_mass_cgs = 9.1093897e-28  # g
electron_charge_cgs = 4.80320425e-10  # statcoulomb
amu_cgs = 1.6605402e-24  # g
bohr_radius_cgs = 5.29177210903e-9  # cm
solar_mass_cgs = 1.9884e33
G_cgs = 6.67430e-8
eV_to_cgs = 1.602e-12
kboltz_eV = 8.617333262145e-5
hplanck_eV = 4.135667696e-15
RydbergH_eV = 13.598287264
Rydberg_eV = 13.605693122994
