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
