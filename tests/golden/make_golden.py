"""Regenerate the golden fixtures from Korg.jl's own test data.

    python tests/golden/make_golden.py /path/to/Korg.jl

lyman_absorption.npz: the reference's hydrogen-line golden vector (test/data/lyman_absorption.h5,
used by test/line_absorption.jl:19-39 with atol 5e-9), its attributes, and the H I partition
function at 9000 K that the reference test evaluates (default_partition_funcs[H I](log 9000)).
The HDF5 file is read with the package's own reader; the numbers are copied unchanged.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", "..", "korg.jl_gb300"))

from korg_gb300 import hdf5lite  # noqa: E402
from korg_gb300.data import default_partition_funcs  # noqa: E402
from korg_gb300.species import parse_species  # noqa: E402

root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("KORG_REFERENCE")
if not root:
    sys.exit("usage: make_golden.py /path/to/Korg.jl  (or set KORG_REFERENCE)")
f = hdf5lite.File(os.path.join(root, "test", "data", "lyman_absorption.h5"))
a = f["profile"].attrs
U = default_partition_funcs()[parse_species("H I")](np.log(9000.0))
np.savez(os.path.join(HERE, "lyman_absorption.npz"), profile=f.read("profile"), T=a["T"], ne=a["ne"],
         nH_I=a["nH_I"], start_wl=a["start_wl"], stop_wl=a["stop_wl"], wl_step=a["wl_step"],
         UH_I_9000=U)
print("wrote lyman_absorption.npz; U(H I, 9000 K) =", U)

# marcs_layers.npz: T, n_tot and n_e of every layer of the reference's three MARCS test
# atmospheres (test/data/*.mod), read with the column layout of src/atmosphere.jl:184-225
# (n = P / kT), and each file's abundance table (A(X), -99 where absent); the inputs of the
# chemical-equilibrium parity tests.
kB = 1.380649e-16
out = {}
for name in ("sun", "s5000_g+3.0_m1.0_t02_st_z+0.00_a+0.00_c+0.00_n+0.00_o+0.00_r+0.00_s+0.00",
             "s6000_g+1.0_m0.5_t05_st_z+0.00_a+0.00_c+0.00_n+0.00_o+0.00_r+0.00_s+0.00"):
    lines = open(os.path.join(root, "test", "data", name + ".mod")).read().split("\n")
    n = int(next(l for l in lines if "Number of depth points" in l).split()[0])
    h = next(i for i, l in enumerate(lines) if "lgTauR" in l)
    a = next(i for i, l in enumerate(lines) if "Logarithmic chemical number abundances" in l)
    A_X = []
    for l in lines[a + 1:]:
        if len(A_X) >= 92:
            break
        A_X += [float(v) for v in l.split()]
    T = np.array([float(l[29:36]) for l in lines[h + 1:h + 1 + n]])
    Pe = np.maximum(np.array([float(l[38:48]) for l in lines[h + 1:h + 1 + n]]), 0)
    Pg = np.maximum(np.array([float(l[48:60]) for l in lines[h + 1:h + 1 + n]]), 0)
    key = name.split("_")[0] if name != "sun" else "sun"
    out[key + "_T"], out[key + "_ne"], out[key + "_n_tot"] = T, Pe / (T * kB), Pg / (T * kB)
    out[key + "_A_X"] = np.array(A_X[:92])
np.savez(os.path.join(HERE, "marcs_layers.npz"), **out)
print("wrote marcs_layers.npz:", sorted(out))
