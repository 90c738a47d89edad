"""Lagrangian parcel files (dsmcParcelIO.C:133-450): reading the reference's
own cloud files (the first 2000 parcels of couette_N2-O2/backup-5, kept in
their file format by tests/golden/make_couette_golden.py), writing a cloud
and reading it back bit for bit, OpenFOAM cell labels of a two-block mesh,
and the errors of malformed files."""
import os
import re
import shutil

import numpy as np
import pytest

from hystrath_gb300 import spec as S

HERE = os.path.dirname(os.path.abspath(__file__))
COUETTE = os.path.join(HERE, "golden", "cases", "couette_N2-O2")
PLATE = os.path.join(HERE, "golden", "cases", "supersonic_flat_plate")
SAMPLE = os.path.join(HERE, "golden", "couette_N2-O2_5_parcels.npz")


def test_reads_the_reference_cloud_files(gpu_lib):
    from hystrath_gb300.dsmc import parse_parcels
    p = parse_parcels(COUETTE, "5", "dsmc")
    ref = np.load(SAMPLE)
    assert len(p["id"]) == 2000
    for k in ("pos", "U", "erot", "species", "vib", "id"):
        np.testing.assert_array_equal(p[k], ref[k].astype(p[k].dtype))
    # the reduced-D coordinate sits at the mesh centre, and the stored cell
    # labels are OpenFOAM's i + 5 j of the positions
    assert np.all(p["pos"][:, 2] == 0.005)
    i = np.floor(p["pos"][:, 0] / 0.01).astype(int)
    j = np.floor(p["pos"][:, 1] / 0.01).astype(int)
    np.testing.assert_array_equal(ref["cell"], i + 5 * j)


def _write_files(d, files):
    os.makedirs(d, exist_ok=True)
    for name, text in files.items():
        with open(os.path.join(d, name), "w") as f:
            f.write("FoamFile { version 2.0; format ascii; class labelField; object %s; }\n" % name + text)


def test_malformed_cloud_files(gpu_lib, tmp_path):
    from hystrath_gb300.dsmc import DsmcError, parse_parcels
    d = tmp_path / "0" / "lagrangian" / "dsmc"
    _write_files(d, {"positions": "2\n(\n(0.1 0.2 0.3) 0\n(0.2 0.2 0.3) 1\n)\n",
                     "U": "2{(1 2 3)}\n", "typeId": "3(0 0 0)\n"})
    with pytest.raises(DsmcError, match="3 entries"):
        parse_parcels(str(tmp_path), "0")
    _write_files(d, {"typeId": "2(0 1)\n", "positions": "1\n(\n(0.25 0.25 0.25 0.25) 0 1 2\n)\n"})
    with pytest.raises(DsmcError, match="barycentric"):
        parse_parcels(str(tmp_path), "0")
    _write_files(d, {"positions": "2\n(\n(0.1 0.2 0.3) 0\n(0.2 0.2 0.3) 1\n)\n"})
    p = parse_parcels(str(tmp_path), "0")     # ERot, vibLevel, origId absent: defaults
    np.testing.assert_array_equal(p["U"], [[1, 2, 3], [1, 2, 3]])
    np.testing.assert_array_equal(p["species"], [0, 1])
    np.testing.assert_array_equal(p["id"], [0, 1])
    assert not p["erot"].any() and not p["vib"].any()
    shutil.rmtree(tmp_path / "0")
    with pytest.raises(DsmcError) as e:
        parse_parcels(str(tmp_path), "0")
    assert e.value.code == S.ERR_IO


def _by_id(p):
    o = np.argsort(p["id"])
    return {k: v[o] for k, v in p.items()}


@pytest.mark.gpu
def test_write_then_read_is_bit_exact(gpu_lib, tmp_path):
    from hystrath_gb300.dsmc import DsmcCloud, parse_case
    case = tmp_path / "plate"
    shutil.copytree(PLATE, case)
    g = DsmcCloud(parse_case(str(case)))
    g.initialise()
    g.evolve(20)
    g.write_parcels(str(case), "0.00008")
    h = DsmcCloud(parse_case(str(case)))
    h.read_parcels(str(case), "0.00008")
    a, b = _by_id(g.particles()), _by_id(h.particles())
    for k in ("pos", "U", "erot", "vib", "species", "id", "cell"):
        np.testing.assert_array_equal(a[k], b[k])
    # the labels are OpenFOAM's: block 0 (5 x 60) first, then block 1 (95 x 60)
    text = open(case / "0.00008" / "lagrangian" / "dsmc" / "positions").read()
    rows = re.findall(r"\(([^()]*)\) (\d+)", text)
    xs = np.array([[float(v) for v in r[0].split()] for r in rows])
    lab = np.array([int(r[1]) for r in rows])
    assert len(lab) == g.info().n_particles
    s = parse_case(str(case))
    xn = np.ctypeslib.as_array(s.node_coords[0], shape=(101,))
    yn = np.ctypeslib.as_array(s.node_coords[1], shape=(61,))
    i = np.searchsorted(xn, xs[:, 0], side="right") - 1
    j = np.searchsorted(yn, xs[:, 1], side="right") - 1
    expect = np.where(i < 5, i + 5 * j, 300 + (i - 5) + 95 * j)
    np.testing.assert_array_equal(lab, expect)


@pytest.mark.gpu
def test_reference_cloud_steps_on_the_gpu(gpu_lib):
    """The reference's parcels (two species, vibrational levels) load into a
    Couette cloud and step; energy changes only through the walls."""
    from hystrath_gb300.dsmc import DsmcCloud, parse_case
    g = DsmcCloud(parse_case(COUETTE))
    g.read_parcels(COUETTE, "5", "dsmc")
    p = _by_id(g.particles())
    ref = np.load(SAMPLE)
    o = np.argsort(ref["id"])
    np.testing.assert_array_equal(p["pos"], ref["pos"][o])
    np.testing.assert_array_equal(p["vib"], ref["vib"][o])
    # sigmaTcRMax comes from the time directory's dsmcSigmaTcRMax
    from tests.test_foam_io import read_foam_field
    sm = read_foam_field(os.path.join(COUETTE, "5", "dsmcSigmaTcRMax"))
    np.testing.assert_array_equal(g.cell_array("sigmaTcRMax"), sm)
    g.evolve(5)
    assert g.info().n_particles == 2000
