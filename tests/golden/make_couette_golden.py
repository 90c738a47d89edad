"""Builds tests/golden/couette_N2-O2_5.npz from the stored outputs of the
reference's couette_N2-O2 tutorial (run/hyStrath/dsmcFoam+/couette_N2-O2/
backup-5 in hystrath/hyStrath).

Those files are dsmcFoam+ fields at t = 5 s (dt 1e-5 s), averaged from
t = 0.5 s on (resetAtOutputUntilTime 0.5).  The mesh is one 5 x 100 x 1 block,
so OpenFOAM's cell order is already i + 5 j.  The fixture keeps each field as
a profile across the channel: the mean over the 5 cells of every row, and
the standard deviation of those 5 cells (their noise); and the mixture's
wall heat flux, shear stress and pressure on the 5 faces of each wall.  The
first 2000 parcels of its lagrangian cloud are kept as files of the same
format (cases/couette_N2-O2/5/lagrangian/dsmc) with their values, beside the
cloud's dsmcSigmaTcRMax field of that time.

Run in a checkout next to the reference:
    python tests/golden/make_couette_golden.py /path/to/hystrath/hyStrath
"""
import os
import re
import shutil
import sys

import numpy as np

NX, NY = 5, 100


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


N_LAGRANGIAN = 2000


def write_lagrangian_sample(src):
    """The first N_LAGRANGIAN parcels of the reference's cloud files, in the
    same file format (header, count, one entry per line), as the case's
    time directory 5/lagrangian/dsmc, with their parsed values beside them."""
    here = os.path.dirname(os.path.abspath(__file__))
    dst = os.path.join(here, "cases", "couette_N2-O2", "5", "lagrangian", "dsmc")
    os.makedirs(dst, exist_ok=True)
    parsed = {}
    for name in ("positions", "U", "ERot", "typeId", "vibLevel", "origId", "newParcel", "origProcId",
                 "classification"):
        text = open(os.path.join(src, name)).read()
        head_end = text.index("}", text.index("FoamFile")) + 1
        head = text[:head_end]
        rest = text[head_end:]
        m = re.search(r"\n(\d+)\s*(\(|\{)", rest)
        n = int(m.group(1))
        if m.group(2) == "{":
            val = re.search(r"\{([^}]*)\}", rest[m.start():]).group(1)
            body = f"\n{N_LAGRANGIAN}{{{val}}}\n"
        else:
            lines = rest[m.end():].lstrip("\n").split("\n")[:N_LAGRANGIAN]
            body = f"\n{N_LAGRANGIAN}\n(\n" + "\n".join(lines) + "\n)\n"
            parsed[name] = lines
        assert n >= N_LAGRANGIAN
        with open(os.path.join(dst, name), "w") as f:
            f.write(head + "\n" + body)
    pos = np.array([[float(v) for v in l[l.index("(") + 1:l.index(")")].split()] for l in parsed["positions"]])
    U = np.array([[float(v) for v in l.strip()[1:-1].split()] for l in parsed["U"]])
    vib = np.array([int(l[l.index("(") + 1:l.index(")")] or 0) for l in parsed["vibLevel"]])
    np.savez_compressed(os.path.join(here, "couette_N2-O2_5_parcels.npz"), pos=pos, U=U,
                        erot=np.array(parsed["ERot"], dtype=float), species=np.array(parsed["typeId"], dtype=int),
                        vib=vib, id=np.array(parsed["origId"], dtype=np.int64),
                        cell=np.array([int(l[l.index(")") + 1:].split()[0]) for l in parsed["positions"]]))


def main():
    # root of the reference tree: first argument, else $HYSTRATH_REFERENCE
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("HYSTRATH_REFERENCE", "")
    if not ref:
        sys.exit(f"usage: python {sys.argv[0]} <reference tree root> (or set HYSTRATH_REFERENCE)")
    d = os.path.join(ref, "run/hyStrath/dsmcFoam+/couette_N2-O2/backup-5")
    out = {}
    for sp in ("N2", "O2", "mixture"):
        for f in ("Ttra", "Trot", "Tvib", "rhoN", "dsmcNMean"):
            v = read_internal(os.path.join(d, f"{f}_{sp}")).reshape(NY, NX)
            out[f"{f}_{sp}"] = v.mean(1)
            out[f"{f}_{sp}_sd"] = v.std(1, ddof=1)
        u = read_internal(os.path.join(d, f"U_{sp}"))[:, 0].reshape(NY, NX)
        out[f"Ux_{sp}"] = u.mean(1)
        out[f"Ux_{sp}_sd"] = u.std(1, ddof=1)
    # wall fields of the mixture on the 5 faces of each wall
    for f in ("wallHeatFlux", "wallShearStress", "p"):
        for w in ("upperWall", "lowerWall"):
            out[f"{f}_{w}"] = read_patch(os.path.join(d, f"{f}_mixture"), w)
    write_lagrangian_sample(os.path.join(d, "lagrangian", "dsmc"))
    # the cloud's sigmaTcRMax field of the same time, read with the parcels
    here = os.path.dirname(os.path.abspath(__file__))
    shutil.copyfile(os.path.join(d, "dsmcSigmaTcRMax"),
                    os.path.join(here, "cases", "couette_N2-O2", "5", "dsmcSigmaTcRMax"))
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "couette_N2-O2_5.npz")
    np.savez_compressed(path, **out)
    print("wrote", path, len(out), "profiles")


if __name__ == "__main__":
    main()
