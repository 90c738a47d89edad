"""Builds tests/golden/hypersonic_corner_0.003.npz from the stored outputs of
the reference's hypersonicCorner tutorial
(run/hyStrath/dsmcFoam+/hypersonicCorner/backup-0.003 in hystrath/hyStrath).

Those files are time-averaged dsmcFoam+ fields at t = 3e-3 s (averaging
restarted at every write until 1.5e-3 s).  OpenFOAM numbers the cells block by
block (block 0: 5 x 18 x 18, block 1: 25 x 18 x 18, i fastest); the fixture
stores them in the Cartesian order i + 30 (j + 18 k) that this library uses.

Run in a checkout next to the reference:
    python tests/golden/make_hypersonic_corner_golden.py /path/to/hystrath/hyStrath
"""
import os
import re
import sys

import numpy as np

NX, NY, NZ = 30, 18, 18
BLOCKS = [(0, 5), (5, 25)]   # (i offset, cells in x) of the two blocks


def read_internal(path):
    text = open(path).read()
    m = re.search(r"internalField\s+nonuniform\s+List<(scalar|vector)>\s*(\d+)\s*\(", text)
    if not m:
        raise ValueError(f"{path}: no nonuniform internalField")
    kind, n = m.group(1), int(m.group(2))
    body = text[m.end():]
    if kind == "scalar":
        vals = np.array(body.split(None, n)[:n], dtype=np.float64)
    else:
        tup = re.findall(r"\(([^()]*)\)", body)[:n]
        vals = np.array([[float(x) for x in t.split()] for t in tup])
    return vals


def to_cartesian(vals):
    out = np.empty_like(vals)
    src = 0
    for i0, nxb in BLOCKS:
        for k in range(NZ):
            for j in range(NY):
                for i in range(nxb):
                    out[(i0 + i) + NX * (j + NY * k)] = vals[src]
                    src += 1
    return out


def main():
    # root of the reference tree: first argument, else $HYSTRATH_REFERENCE
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("HYSTRATH_REFERENCE", "")
    if not ref:
        sys.exit(f"usage: python {sys.argv[0]} <reference tree root> (or set HYSTRATH_REFERENCE)")
    d = os.path.join(ref, "run/hyStrath/dsmcFoam+/hypersonicCorner/backup-0.003")
    fields = {}
    for name in ("rhoN_Ar", "rhoM_Ar", "Ttra_Ar", "p_Ar", "U_Ar", "dsmcSigmaTcRMax", "dsmcNMean_Ar", "mfp_Ar",
                 "Ma_Ar"):
        v = to_cartesian(read_internal(os.path.join(d, name)))
        fields[name] = v.astype(np.float32)
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "hypersonic_corner_0.003.npz")
    np.savez_compressed(out, **fields)
    print("wrote", out, {k: v.shape for k, v in fields.items()})


if __name__ == "__main__":
    main()
