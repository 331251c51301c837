"""Convert the Korg.jl data tables this package needs into compact .npz files.

Run once, from a checkout that has Korg.jl's ``data/`` directory:

    python make_data.py /path/to/Korg.jl

It reads (with the package's own HDF5 reader, no h5py needed):
  * data/Stehle-Hutchson-hydrogen-profiles.h5  -> stark_profiles.npz
  * data/atomic_partition_funcs/partition_funcs.h5 and
    data/barklem_collet_2016/BarklemCollet2016-molecular_partition.dat -> partition_funcs.npz
  * data/barklem_collet_2016/BarklemCollet2016-ionization_energies.dat -> in partition_funcs.npz
  * data/linelists/alpha_5000/alpha_5000_lines.csv -> alpha_5000_lines.npz
  * the continuum-absorption tables -> continuum_tables.npz: the H I bound-free cross-sections
    (data/bf_cross-sections/individual_H_cross-sections.h5, levels 1-6), the H- bound-free
    cross-sections (data/McLaughlin2017Hminusbf.h5), the free-free Gaunt factors
    (data/vanHoof2014-nr-gauntff.dat, cut to the reference's T / wavelength / Z range), and the
    tables written as array literals in src/ContinuumAbsorption/*.jl (H- ff of Bell & Berrington
    1987, He- ff of John 1994, H2+ of Stancil 1994, departure coefficients of Peach 1970)
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


def _julia_array(src, name, start=0):
    """The numbers of the Julia array literal assigned to `name` (first one at or after `start`),
    as a float array: a matrix literal (rows separated by newlines or ';') gives a 2-D array.  A
    scalar factor written before it (`10.0 .* [...]`) is applied."""
    import re
    m = re.compile(r"\b" + re.escape(name) + r"\s*=\s*([-+0-9.eE]+\s*\.\*\s*)?\[").search(src, start)
    if not m:
        raise KeyError(name)
    i, depth = m.end(), 1
    j = i
    while depth:
        depth += {"[": 1, "]": -1}.get(src[j], 0)
        j += 1
    body = "\n".join(line.split("#")[0] for line in src[i:j - 1].split("\n"))
    rows = [r for r in re.split(r"[;\n]", body) if r.strip()]
    vals = [[float(x) for x in re.split(r"[,\s]+", r.strip()) if x] for r in rows]
    arr = np.array(vals) if len(vals) > 1 and len({len(v) for v in vals}) == 1 and len(vals[0]) > 1 else \
        np.array([x for v in vals for x in v])
    if m.group(1):
        arr = arr * float(m.group(1).split(".*")[0])
    return arr


def continuum(root):
    src_dir = os.path.join(root, "src", "ContinuumAbsorption")
    read = lambda fn: open(os.path.join(src_dir, fn)).read()
    out = {}
    # H I bound-free (Nahar 2021), levels n = 1..6 (absorption_H.jl:9-19, :62 uses [1:n_max_MHD])
    f = hdf5lite.File(os.path.join(root, "data", "bf_cross-sections", "individual_H_cross-sections.h5"))
    n = f.read("n")
    assert list(n[:6]) == [1, 2, 3, 4, 5, 6]
    out["H_bf_E"], out["H_bf_sigma"] = f.read("E")[:6], f.read("sigma")[:6]  # eV, megabarn
    # H- bound-free (McLaughlin 2017, absorption_H.jl:170-175)
    f = hdf5lite.File(os.path.join(root, "data", "McLaughlin2017Hminusbf.h5"))
    out["Hminus_bf_nu"], out["Hminus_bf_sigma"] = f.read("nu"), f.read("sigma")
    # H- free-free (Bell & Berrington 1987, absorption_H.jl:232-259): K in 1e-26 cm^4/dyn
    s = read("absorption_H.jl")
    out["Hminus_ff_theta"] = _julia_array(s, "theta_ff_absorption_interp")
    out["Hminus_ff_lambda"] = _julia_array(s, "lambda_ff_absorption_interp")
    out["Hminus_ff_K"] = _julia_array(s, "ff_absorption")
    # He- free-free (John 1994, absorption_He.jl:31-53)
    s = read("absorption_He.jl")
    out["Heminus_ff_theta"] = _julia_array(s, "theta_ff_absorption_interp")
    out["Heminus_ff_lambda"] = _julia_array(s, "lambda_ff_absorption_interp")
    out["Heminus_ff_K"] = _julia_array(s, "ff_absorption")
    # H2+ (Stancil 1994): K(T) n(H I) n(H II) / n(H2+), cross sections in 1e-18 cm^2 (bf) and
    # 1e-39 cm^5 (ff) on wavelengths in A (Stancil1994.jl)
    s = read("Stancil1994.jl")
    for k in ("Ts_H2plus", "K_H2plus_vals", "λs_H2plus_ff", "λs_bf", "σ_H2plus_bf_table", "σ_H2plus_ff_table"):
        key = {"λs_H2plus_ff": "H2plus_ff_lambda", "λs_bf": "H2plus_bf_lambda", "σ_H2plus_bf_table": "H2plus_bf_sigma",
               "σ_H2plus_ff_table": "H2plus_ff_sigma", "Ts_H2plus": "H2plus_T", "K_H2plus_vals": "H2plus_K"}[k]
        out[key] = _julia_array(s, k)
    # Peach 1970 ff departure coefficients, per ion taking part (Peach1970.jl)
    s = read("Peach1970.jl")
    for sp in ("He II", "C II", "Si II", "Mg II"):
        at = s.index(f'coeffs[species"{sp}"] = let')
        tag = sp.replace(" ", "")
        out[f"peach_{tag}_sigma"] = _julia_array(s, "σ_vals", at)
        out[f"peach_{tag}_T"] = _julia_array(s, "T_vals", at)
        out[f"peach_{tag}_D"] = _julia_array(s, "table_vals", at)
    # van Hoof et al. (2014) non-relativistic thermally averaged ff Gaunt factors
    # (hydrogenic_bf_ff.jl:16-80): the header gives the grid, rows are log10(u), columns log10(gamma^2)
    lines = [l for l in open(os.path.join(root, "data", "vanHoof2014-nr-gauntff.dat"))]
    body = [l for l in lines if not l.startswith("#")]
    hdr = lambda l: l.split("#")[0].split()
    assert int(hdr(body[0])[0]) == 20140210
    n_g2, n_u = (int(x) for x in hdr(body[1]))
    g2_start, u_start, step = float(hdr(body[2])[0]), float(hdr(body[3])[0]), float(hdr(body[4])[0])
    tab = np.array([[float(x) for x in body[5 + i].split()] for i in range(n_u)])
    log_g2 = g2_start + step * np.arange(n_g2)
    log_u = u_start + step * np.arange(n_u)
    Ry, kB, h, c = 13.605693122994, 8.617333262145e-5, 6.62607015e-27, 2.99792458e10
    kB_cgs = 1.380649e-16
    g2 = [np.log10(Ry * Z * Z / (kB * T)) for Z in (1, 2) for T in (100.0, 1e6)]
    uu = [np.log10(h * c / (lam * kB_cgs * T)) for lam in (1e-6, 1e-2) for T in (100.0, 1e6)]
    g_lb, g_ub = np.searchsorted(log_g2, min(g2), "right") - 1, np.searchsorted(log_g2, max(g2), "left")
    u_lb, u_ub = np.searchsorted(log_u, min(uu), "right") - 1, np.searchsorted(log_u, max(uu), "left")
    out["gaunt_log_u"], out["gaunt_log_g2"] = log_u[u_lb:u_ub + 1], log_g2[g_lb:g_ub + 1]
    out["gaunt_ff"] = tab[u_lb:u_ub + 1, g_lb:g_ub + 1]
    np.savez_compressed(os.path.join(HERE, "continuum_tables.npz"), **out)


def _julia_nested_dict(src, name):
    """``name = Dict(Z => Dict(A => v, ...), ...)`` as {Z: {A: v}} (src/isotopic_data.jl)."""
    import re
    start = src.index(name)
    i = src.index("Dict(", start) + 5
    depth, j = 1, i
    while depth:
        depth += {"(": 1, ")": -1}.get(src[j], 0)
        j += 1
    body = "\n".join(line.split("#")[0] for line in src[i:j - 1].split("\n"))
    out = {}
    for z, inner in re.findall(r"(\d+)\s*=>\s*Dict\(([^)]*)\)", body):
        out[int(z)] = {int(a): float(v) for a, v in re.findall(r"(\d+)\s*=>\s*([-+0-9.eE]+)", inner)}
    return out


def equilibrium(root):
    """Molecular equilibrium constants (src/read_statmech_quantities.jl:53-130, 203-226):
    Barklem & Collet log10 K tables (molecule names, ln T knots, log10 K, as stored), the ExoMol
    polyatomic partition functions (T, U as stored) with the nuclear-spin degeneracy of each
    molecule's most abundant isotopologue, and the polyatomic atomization energies (kJ/mol)."""
    f = hdf5lite.File(os.path.join(root, "data", "barklem_collet_2016", "barklem_collet_ks.h5"))
    mols = [str(m) for m in f.read("mols")]
    lnTs, logKs = f.read("lnTs").T.copy(), f.read("logKs").T.copy()  # file order is (T, molecule)
    g = hdf5lite.File(os.path.join(root, "data", "polyatomic_partition_funcs", "polyatomic_partition_funcs.h5"))
    poly, T, U, off = sorted(g.keys()), [], [], [0]
    for name in poly:
        T.append(g.read(name + "/temp"))
        U.append(g.read(name + "/partition_function"))
        off.append(off[-1] + len(T[-1]))
    iso = open(os.path.join(root, "src", "isotopic_data.jl")).read()
    abund = _julia_nested_dict(iso, "isotopic_abundances")
    spin = _julia_nested_dict(iso, "isotopic_nuclear_spin_degeneracies")
    g_ns = []
    for name in poly:  # product over atoms of the most abundant isotope's degeneracy (:211-219)
        prod = 1.0
        for Z in parse_species(name).atoms:
            A = max(abund[Z], key=abund[Z].get)
            prod *= spin[Z][A]
        g_ns.append(prod)
    rows = list(csv.DictReader(open(os.path.join(root, "data", "polyatomic_partition_funcs",
                                                 "atomization_energies.csv"))))
    np.savez_compressed(
        os.path.join(HERE, "equilibrium_constants.npz"),
        bc_mols=np.array(mols), bc_lnTs=lnTs, bc_logKs=logKs,
        poly_names=np.array(poly), poly_T=np.concatenate(T), poly_U=np.concatenate(U),
        poly_off=np.array(off, np.int64), poly_g_ns=np.array(g_ns),
        atomization_names=np.array([r["spec"] for r in rows]),
        atomization_kJmol=np.array([float(r["energy"]) for r in rows]))


if __name__ == "__main__":
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("KORG_REFERENCE")
    if not root:
        sys.exit("usage: make_data.py /path/to/Korg.jl  (or set KORG_REFERENCE)")
    stark(root)
    partition(root)
    alpha5000(root)
    continuum(root)
    equilibrium(root)
    print("wrote", sorted(x for x in os.listdir(HERE) if x.endswith(".npz")))
