"""OpenFOAM-format field output (dsmcVolFields::writeField): the written
files parse back to the library's fields in OpenFOAM's blockMesh cell order."""
import os
import re
import shutil

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CASE = os.path.join(HERE, "golden", "cases", "hypersonic_corner")


def read_foam_field(path):
    text = open(path).read()
    m = re.search(r"internalField\s+nonuniform\s+List<(scalar|vector)>\s*(\d+)\s*\(", text)
    assert m, path
    kind, n = m.group(1), int(m.group(2))
    body = text[m.end():]
    if kind == "scalar":
        return np.array(body.split(None, n)[:n], dtype=np.float64)
    tup = re.findall(r"\(([^()]*)\)", body)[:n]
    return np.array([[float(x) for x in t.split()] for t in tup])


def block_order():
    # hypersonicCorner blockMeshDict: block 0 is 5 x 18 x 18 at i = 0,
    # block 1 is 25 x 18 x 18 at i = 5 (i fastest within a block)
    order = []
    for i0, nxb in ((0, 5), (5, 25)):
        for k in range(18):
            for j in range(18):
                for i in range(nxb):
                    order.append((i0 + i) + 30 * (j + 18 * k))
    return np.array(order)


@pytest.mark.gpu
def test_fields_written_in_blockmesh_order(tmp_path):
    from hystrath_gb300.dsmc import DsmcCloud
    case = tmp_path / "case"
    shutil.copytree(CASE, case)
    g = DsmcCloud(str(case))
    g.initialise()
    g.evolve(20)
    g.write_fields(str(case), "2e-05", "Ar")
    order = block_order()
    for name in ("rhoN", "Ttra", "p", "dsmcNMean"):
        got = read_foam_field(str(case / "2e-05" / f"{name}_Ar"))
        np.testing.assert_allclose(got, g.field(name)[order], rtol=1e-9, atol=0)
    U = read_foam_field(str(case / "2e-05" / "U_Ar"))
    np.testing.assert_allclose(U[:, 0], g.field("Ux")[order], rtol=1e-9, atol=1e-12)
    smax = read_foam_field(str(case / "2e-05" / "dsmcSigmaTcRMax"))
    np.testing.assert_allclose(smax, g.cell_array("sigmaTcRMax")[order], rtol=1e-9)
    text = open(case / "2e-05" / "Ttra_Ar").read()
    assert "class       volScalarField;" in text and "boundaryField" in text
