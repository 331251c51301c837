"""Convert the Korg.jl data tables this package needs into compact .npz files.

Run once, from a checkout that has Korg.jl's ``data/`` directory:

    python make_data.py /path/to/Korg.jl

It reads (with the package's own HDF5 reader, no h5py needed):
  * data/Stehle-Hutchson-hydrogen-profiles.h5  -> stark_profiles.npz
  * data/atomic_partition_funcs/partition_funcs.h5 and
    data/barklem_collet_2016/BarklemCollet2016-molecular_partition.dat -> partition_funcs.npz
  * data/barklem_collet_2016/BarklemCollet2016-ionization_energies.dat -> in partition_funcs.npz
  * data/linelists/alpha_5000/alpha_5000_lines.csv -> alpha_5000_lines.npz
The outputs are the same numbers in a different container; nothing is refitted.
"""
import csv
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from korg_gb300 import hdf5lite  # noqa: E402
from korg_gb300.species import parse_species  # noqa: E402


def stark(root):
    f = hdf5lite.File(os.path.join(root, "data", "Stehle-Hutchson-hydrogen-profiles.h5"))
    names = f.keys()  # file (name) order, as Korg's map(keys(fid)) iterates
    out = {k: [] for k in ["temps", "nes", "dnu", "profile", "lambda0"]}
    meta = {k: [] for k in ["lower", "upper", "Kalpha", "log_gf", "nT", "nNe", "nD"]}
    for n in names:
        g = f[n]
        T = f.read(n + "/temps")
        ne = f.read(n + "/electron_number_densities")
        d = f.read(n + "/delta_nu_over_F0")
        P = f.read(n + "/profile")  # (nD, nNe, nT) in file order
        l0 = f.read(n + "/lambda0")  # (nNe, nT)
        assert P.shape == (len(d), len(ne), len(T)) and l0.shape == (len(ne), len(T))
        out["temps"].append(T)
        out["nes"].append(ne)
        out["dnu"].append(d)
        out["profile"].append(P.ravel())
        out["lambda0"].append(l0.ravel())
        for k in ["lower", "upper", "Kalpha", "log_gf"]:
            meta[k].append(g.attrs[k])
        meta["nT"].append(len(T))
        meta["nNe"].append(len(ne))
        meta["nD"].append(len(d))
    arrs = {k: np.concatenate(v) for k, v in out.items()}
    arrs.update({k: np.asarray(v) for k, v in meta.items()})
    arrs["names"] = np.array(names)
    np.savez_compressed(os.path.join(HERE, "stark_profiles.npz"), **arrs)


def partition(root):
    f = hdf5lite.File(os.path.join(root, "data", "atomic_partition_funcs", "partition_funcs.h5"))
    logT_min, logT_step, logT_max = f.read("logT_min"), f.read("logT_step"), f.read("logT_max")
    atomic = sorted(k for k in f.keys() if not k.startswith("logT"))
    U_atomic = np.stack([f.read(k) for k in atomic])
    # molecular partition functions (text table, temperatures in the '# T [K]' header line)
    temps, mols, U_mol = [], [], []
    path = os.path.join(root, "data", "barklem_collet_2016", "BarklemCollet2016-molecular_partition.dat")
    for line in open(path):
        if len(line) >= 9 and "T [K]" in line:
            temps += [float(x) for x in line[9:].split()]
        elif line.startswith("#"):
            continue
        else:
            toks = line.split()
            if not toks or toks[0].startswith("D_"):
                continue
            mols.append(toks[0])
            U_mol.append([float(x) for x in toks[1:]])
    ion = {}
    path = os.path.join(root, "data", "barklem_collet_2016", "BarklemCollet2016-ionization_energies.dat")
    for line in open(path):
        if line[0] != "#":
            t = line.split()
            ion[int(t[0])] = [float(x) for x in t[2:]]
    Z = sorted(ion)
    np.savez_compressed(
        os.path.join(HERE, "partition_funcs.npz"),
        logT_min=logT_min, logT_step=logT_step, logT_max=logT_max,
        atomic_names=np.array(atomic), U_atomic=U_atomic,
        mol_temps=np.array(temps), mol_names=np.array(mols), U_mol=np.array(U_mol),
        ion_Z=np.array(Z), ion_E=np.array([ion[z] for z in Z]))


def alpha5000(root):
    path = os.path.join(root, "data", "linelists", "alpha_5000", "alpha_5000_lines.csv")
    rows = list(csv.DictReader(open(path)))
    vdW = []
    for r in rows:
        v = r["vdW"]
        if "," in v:
            a, b = v.strip("()").split(",")
            vdW.append((float(a), float(b)))
        else:
            vdW.append((float(v), np.nan))  # a single float: converted by the Line rules
    np.savez_compressed(
        os.path.join(HERE, "alpha_5000_lines.npz"),
        wl=np.array([float(r["wl"]) for r in rows]),
        log_gf=np.array([float(r["log_gf"]) for r in rows]),
        species=np.array([str(parse_species(r["species"])) for r in rows]),
        E_lower=np.array([float(r["E_lower"]) for r in rows]),
        gamma_rad=np.array([float(r["gamma_rad"]) for r in rows]),
        gamma_stark=np.array([float(r["gamma_stark"]) for r in rows]),
        vdW=np.array(vdW))


if __name__ == "__main__":
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("KORG_REFERENCE")
    if not root:
        sys.exit("usage: make_data.py /path/to/Korg.jl  (or set KORG_REFERENCE)")
    stark(root)
    partition(root)
    alpha5000(root)
    print("wrote", sorted(x for x in os.listdir(HERE) if x.endswith(".npz")))
