"""Species bookkeeping for the host side: names, masses and the molecule flag.

Korg identifies a species by a formula (atoms sorted by atomic number) and a charge
(src/species.jl:181-307).  Here a species is the tuple ``(atoms, charge)`` with ``atoms`` a
sorted tuple of atomic numbers.  Masses are standard atomic weights in amu (the same
four-significant-figure table Korg uses, src/atomic_data.jl:16-26) times the amu in grams.
"""
from __future__ import annotations

import re

from .constants import amu_cgs

atomic_symbols = [
    "H", "He", "Li", "Be", "B", "C", "N", "O", "F", "Ne", "Na", "Mg", "Al", "Si", "P", "S", "Cl",
    "Ar", "K", "Ca", "Sc", "Ti", "V", "Cr", "Mn", "Fe", "Co", "Ni", "Cu", "Zn", "Ga", "Ge", "As",
    "Se", "Br", "Kr", "Rb", "Sr", "Y", "Zr", "Nb", "Mo", "Tc", "Ru", "Rh", "Pd", "Ag", "Cd", "In",
    "Sn", "Sb", "Te", "I", "Xe", "Cs", "Ba", "La", "Ce", "Pr", "Nd", "Pm", "Sm", "Eu", "Gd", "Tb",
    "Dy", "Ho", "Er", "Tm", "Yb", "Lu", "Hf", "Ta", "W", "Re", "Os", "Ir", "Pt", "Au", "Hg", "Tl",
    "Pb", "Bi", "Po", "At", "Rn", "Fr", "Ra", "Ac", "Th", "Pa", "U"]
atomic_numbers = {s: i + 1 for i, s in enumerate(atomic_symbols)}

_weights_amu = [
    1.008, 4.003, 6.941, 9.012, 10.81, 12.01, 14.01, 16.00, 19.00, 20.18, 22.99, 24.31, 26.98,
    28.08, 30.97, 32.06, 35.45, 39.95, 39.10, 40.08, 44.96, 47.90, 50.94, 52.00, 54.94, 55.85,
    58.93, 58.71, 63.55, 65.37, 69.72, 72.59, 74.92, 78.96, 79.90, 83.80, 85.47, 87.62, 88.91,
    91.22, 92.91, 95.94, 98.91, 101.1, 102.9, 106.4, 107.9, 112.4, 114.8, 118.7, 121.8, 127.6,
    126.9, 131.3, 132.9, 137.3, 138.9, 140.1, 140.9, 144.2, 145.0, 150.4, 152.0, 157.3, 158.9,
    162.5, 164.9, 167.3, 168.9, 173.0, 175.0, 178.5, 181.0, 183.9, 186.2, 190.2, 192.2, 195.1,
    197.0, 200.6, 204.4, 207.2, 209.0, 210.0, 210.0, 222.0, 223.0, 226.0, 227.0, 232.0, 231.0,
    238.0]
atomic_masses = [w * amu_cgs for w in _weights_amu]

_roman = ["I", "II", "III", "IV", "V"]


class Species(tuple):
    """``Species(atoms, charge)``; construct from text with :func:`parse_species`."""

    def __new__(cls, atoms, charge=0):
        return super().__new__(cls, (tuple(sorted(atoms)), int(charge)))

    def __reduce__(self):  # pickles as Species(atoms, charge)
        return (Species, (self[0], self[1]))

    @property
    def atoms(self):
        return self[0]

    @property
    def charge(self):
        return self[1]

    def ismolecule(self):
        return len(self.atoms) > 1

    def mass(self):
        return sum(atomic_masses[z - 1] for z in self.atoms)

    def __str__(self):
        if self.ismolecule():
            out = "".join(atomic_symbols[z - 1] for z in self.atoms)
            return out + ("+" if self.charge == 1 else "")
        if self.charge < 0:
            return atomic_symbols[self.atoms[0] - 1] + "-" * -self.charge
        return f"{atomic_symbols[self.atoms[0] - 1]} {_roman[self.charge]}"

    __repr__ = __str__


def parse_species(code: str) -> Species:
    """Parse 'Fe I', 'Fe_II', 'Fe 2', 'CO', 'OTi', 'H2', 'H2+' (src/species.jl Species(str))."""
    s = code.strip().replace("_", " ")
    charge = 0
    parts = s.split()
    if len(parts) == 2:
        s, ion = parts
        if ion in _roman:
            charge = _roman.index(ion)
        else:
            charge = int(ion) - 1 if ion.isdigit() else 0
    elif s.endswith("+"):
        s, charge = s[:-1], 1
    elif s.endswith("-"):
        s, charge = s[:-1], -1
    atoms = []
    for sym, count in re.findall(r"([A-Z][a-z]?)(\d*)", s):
        atoms += [atomic_numbers[sym]] * (int(count) if count else 1)
    if not atoms:
        raise ValueError(f"cannot parse species {code!r}")
    return Species(atoms, charge)
