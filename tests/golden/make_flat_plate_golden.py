"""Builds tests/golden/supersonic_flat_plate_0.04.npz from the stored outputs
of the reference's supersonicFlatPlate tutorial
(run/hyStrath/dsmcFoam+/supersonicFlatPlate/backup-0.04 in hystrath/hyStrath).

Those files are dsmcFoam+ fields at t = 0.04 s (dt 4e-6 s), averaged from
t = 8e-3 s on.  OpenFOAM numbers the cells block by block (block 0: 5 x 60,
block 1: 95 x 60, i fastest); the fixture stores them in the Cartesian order
i + 100 j that this library uses, with the plate's wall fields (95 faces,
x from 50 mm on) in x order.

Run in a checkout next to the reference:
    python tests/golden/make_flat_plate_golden.py /path/to/hystrath/hyStrath
"""
import os
import re
import sys

import numpy as np

NX, NY = 100, 60
BLOCKS = [(0, 5), (5, 95)]   # (i offset, cells in x) of the two blocks


def read_internal(path):
    text = open(path).read()
    m = re.search(r"internalField\s+nonuniform\s+List<(scalar|vector)>\s*(\d+)\s*\(", text)
    if not m:
        raise ValueError(f"{path}: no nonuniform internalField")
    kind, n = m.group(1), int(m.group(2))
    body = text[m.end():]
    if kind == "scalar":
        return np.array(body.split(None, n)[:n], dtype=np.float64)
    tup = re.findall(r"\(([^()]*)\)", body)[:n]
    return np.array([[float(x) for x in t.split()] for t in tup])


def read_patch(path, patch):
    text = open(path).read()
    text = text[text.index("boundaryField"):]
    m = re.search(patch + r"\s*\{[^}]*?value\s+nonuniform\s+List<scalar>\s*(\d+)\s*\(([^)]*)\)", text)
    if not m:
        raise ValueError(f"{path}: no values on {patch}")
    return np.array(m.group(2).split(), dtype=np.float64)


def to_cartesian(vals):
    out = np.empty_like(vals)
    src = 0
    for i0, nxb in BLOCKS:
        for j in range(NY):
            for i in range(nxb):
                out[(i0 + i) + NX * j] = vals[src]
                src += 1
    return out


def main():
    # root of the reference tree: first argument, else $HYSTRATH_REFERENCE
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("HYSTRATH_REFERENCE", "")
    if not ref:
        sys.exit(f"usage: python {sys.argv[0]} <reference tree root> (or set HYSTRATH_REFERENCE)")
    d = os.path.join(ref, "run/hyStrath/dsmcFoam+/supersonicFlatPlate/backup-0.04")
    out = {}
    for name in ("rhoN", "Ttra", "Trot", "p", "dsmcNMean"):
        out[name] = to_cartesian(read_internal(os.path.join(d, f"{name}_N2cold"))).astype(np.float32)
    U = to_cartesian(read_internal(os.path.join(d, "U_N2cold")))
    out["Ux"] = U[:, 0].astype(np.float32)
    out["Uy"] = U[:, 1].astype(np.float32)
    for f in ("wallHeatFlux", "wallShearStress", "p"):
        out[f"{f}_plate"] = read_patch(os.path.join(d, f"{f}_N2cold"), "plate")
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "supersonic_flat_plate_0.04.npz")
    np.savez_compressed(path, **out)
    print("wrote", path, {k: v.shape for k, v in out.items()})


if __name__ == "__main__":
    main()
