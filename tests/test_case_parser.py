"""The OpenFOAM case reader behind dsmc_create(case_dir): dictionaries of the
dsmcFoam+ tutorials, blockMeshDict geometry, runtime-selection names and the
reference's error behaviour for unknown models (BinaryCollisionModel.C:72-83,
collisionPartnerSelection.C:82-91, dsmcPatchBoundary.C:79-85)."""
import ctypes as C
import os
import shutil

import numpy as np
import pytest

from hystrath_gb300 import spec as S

HERE = os.path.dirname(os.path.abspath(__file__))
CASE = os.path.join(HERE, "golden", "cases", "hypersonic_corner")
# the reference tree, when present, via HYSTRATH_REFERENCE (its root directory)
REF_ROOT = os.environ.get("HYSTRATH_REFERENCE", "")
REF_CASE = os.path.join(REF_ROOT, "run/hyStrath/dsmcFoam+/hypersonicCorner") if REF_ROOT else ""


def parse(path):
    from hystrath_gb300.dsmc import parse_case
    return parse_case(path)


def face_maps(s):
    out = []
    for q in range(6):
        a = q // 2
        b, c = (1 if a == 0 else 0), (1 if a == 2 else 2)
        n = s.n_cells[b] * s.n_cells[c]
        out.append(np.ctypeslib.as_array(s.face_patch[q], shape=(n,)).copy())
    return out


def test_parse_corner_case(gpu_lib):
    s = parse(CASE)
    assert list(s.n_cells) == [30, 18, 18]
    assert np.allclose(list(s.cell_size), [0.01] * 3)
    assert s.n_species == 1 and s.species[0].name == b"Ar"
    assert s.species[0].mass == 66.3e-27 and s.species[0].omega == 0.81
    assert s.n_equivalent_particles == 0.6e12 and s.delta_t == 1e-6
    assert s.binary_collision_model == S.COLL_VHS and s.partner_selection_model == S.SEL_NTC
    names = [s.patches[p].name for p in range(s.n_patches)]
    assert names == [b"flow", b"entrance", b"walls"]
    flow, ent, walls = (s.patches[p] for p in range(3))
    assert flow.type == S.PATCH_PATCH and flow.model == S.BC_DELETION and flow.inflow == 1
    assert flow.inflow_number_density[0] == 1e20 and flow.inflow_t_tra == 300 and flow.inflow_velocity[0] == 1936
    assert ent.type == S.PATCH_SYMMETRY
    assert walls.type == S.PATCH_WALL and walls.model == S.BC_DIFFUSE and walls.wall_temperature == 1000
    fm = face_maps(s)
    # y = 0 side: symmetry for x < 5 cells, wall downstream
    y0 = fm[2].reshape(18, 30)
    assert np.all(y0[:, :5] == 1) and np.all(y0[:, 5:] == 2)
    assert np.all(fm[0] == 0) and np.all(fm[1] == 0) and np.all(fm[3] == 0)
    assert s.init_number_density[0] == 1e20 and s.init_velocity[0] == 1936
    assert s.measure_mean_free_path == 1 and s.n_obstacles == 0


@pytest.mark.skipif(not REF_CASE or not os.path.isdir(REF_CASE),
                    reason="HYSTRATH_REFERENCE does not name a reference tree")
def test_reference_tutorial_parses_to_the_same_case(gpu_lib):
    """The reference's own hypersonicCorner dictionaries (old 'patches'
    syntax, no ';' after the list) resolve to the same case."""
    a, b = parse(CASE), parse(REF_CASE)
    for k in ("n_cells", "cell_size", "origin"):
        assert list(getattr(a, k)) == pytest.approx(list(getattr(b, k)))
    assert a.n_patches == b.n_patches
    for p in range(a.n_patches):
        pa, pb = a.patches[p], b.patches[p]
        assert (pa.name, pa.type, pa.model, pa.inflow, pa.wall_temperature) == \
               (pb.name, pb.type, pb.model, pb.inflow, pb.wall_temperature)
    for x, y in zip(face_maps(a), face_maps(b)):
        np.testing.assert_array_equal(x, y)
    assert a.n_equivalent_particles == b.n_equivalent_particles and a.delta_t == b.delta_t
    assert bytes(a.species[0]) == bytes(b.species[0])


def _copy_case(tmp_path):
    d = tmp_path / "case"
    shutil.copytree(CASE, d)
    return d


def _edit(path, old, new):
    t = open(path).read()
    assert old in t
    open(path, "w").write(t.replace(old, new))


def _expect(tmp_case, code, needle):
    from hystrath_gb300.dsmc import DsmcError
    with pytest.raises(DsmcError) as e:
        parse(str(tmp_case))
    assert e.value.code == code, str(e.value)
    assert needle in str(e.value)


def test_unknown_binary_collision_model(gpu_lib, tmp_path):
    d = _copy_case(tmp_path)
    _edit(d / "constant/dsmcProperties", "VariableHardSphere;", "GeneralisedHardSphere;")
    _expect(d, S.ERR_UNKNOWN_MODEL, "Valid BinaryCollisionModel types are: 4(VariableHardSphere "
                                    "LarsenBorgnakkeVariableHardSphere VariableSoftSphere "
                                    "LarsenBorgnakkeVariableSoftSphere)")


def test_soft_sphere_models_are_selected_by_name(gpu_lib, tmp_path):
    from hystrath_gb300.dsmc import parse_case
    for name, code in (("VariableSoftSphere", S.COLL_VSS), ("LarsenBorgnakkeVariableSoftSphere", S.COLL_LB_VSS)):
        d = _copy_case(tmp_path / name)
        _edit(d / "constant/dsmcProperties", "VariableHardSphere;", name + ";")
        assert parse_case(str(d)).binary_collision_model == code


def test_unknown_partner_selection(gpu_lib, tmp_path):
    d = _copy_case(tmp_path)
    _edit(d / "constant/dsmcProperties", "noTimeCounter;", "noRepeatCollisions;")
    _expect(d, S.ERR_UNKNOWN_MODEL, "2(noTimeCounter simplifiedBernoulliTrials)")


def test_bernoulli_trials_selected_by_name(gpu_lib, tmp_path):
    d = _copy_case(tmp_path)
    _edit(d / "constant/dsmcProperties", "noTimeCounter;", "simplifiedBernoulliTrials;")
    assert parse(str(d)).partner_selection_model == S.SEL_SBT


def test_unknown_patch_model(gpu_lib, tmp_path):
    d = _copy_case(tmp_path)
    _edit(d / "system/boundariesDict", "boundaryModel dsmcDiffuseWallPatch;", "boundaryModel dsmcCLLWallPatch;")
    _expect(d, S.ERR_UNKNOWN_MODEL, "dsmcSpecularWallPatch dsmcDiffuseWallPatch dsmcDeletionPatch")


def test_missing_patch_in_boundaries(gpu_lib, tmp_path):
    d = _copy_case(tmp_path)
    _edit(d / "system/boundariesDict", "patchName walls;", "patchName wallz;")
    _expect(d, S.ERR_INVALID, "Cannot find patch: wallz")


def test_graded_block_gives_node_coordinates(gpu_lib, tmp_path):
    """simpleGrading ratio r over n cells: widths grow geometrically with
    last / first = r (blockMesh lineDivide); the other block stays uniform,
    so x becomes a graded axis and y, z stay uniform."""
    d = _copy_case(tmp_path)
    _edit(d / "system/blockMeshDict", "(5 18 18) simpleGrading (1 1 1)", "(5 18 18) simpleGrading (2 1 1)")
    s = parse(str(d))
    assert list(s.n_cells) == [30, 18, 18]
    assert bool(s.node_coords[0]) and not s.node_coords[1] and not s.node_coords[2]
    x = np.ctypeslib.as_array(s.node_coords[0], shape=(31,))
    w = np.diff(x)
    assert w[4] / w[0] == pytest.approx(2.0) and np.allclose(w[1:5] / w[:4], 2.0 ** 0.25)
    assert x[5] == pytest.approx(0.05) and np.allclose(w[5:], 0.01)


def test_reversed_block_grading(gpu_lib, tmp_path):
    """A block whose vertex 0 sits at its +x corner grades from that corner."""
    d = _copy_case(tmp_path)
    _edit(d / "system/blockMeshDict", "hex (0 1 2 3 4 5 6 7) (5 18 18) simpleGrading (1 1 1)",
          "hex (1 0 4 5 2 3 7 6) (5 18 18) simpleGrading (2 1 1)")
    s = parse(str(d))
    w = np.diff(np.ctypeslib.as_array(s.node_coords[0], shape=(31,)))
    assert w[0] / w[4] == pytest.approx(2.0)


def test_blocks_that_do_not_meet_node_to_node(gpu_lib, tmp_path):
    d = _copy_case(tmp_path)
    _edit(d / "system/blockMeshDict", "(5 18 18) simpleGrading (1 1 1)", "(5 18 18) simpleGrading (1 2 1)")
    _expect(d, S.ERR_INVALID, "face to face")


def test_unlisted_faces_go_to_an_empty_default_patch(gpu_lib, tmp_path):
    """blockMesh's defaultFaces: here the z sides, one cell thick."""
    d = _copy_case(tmp_path)
    t = open(d / "system/blockMeshDict").read()
    t = t.replace("(5 18 18) simpleGrading", "(5 18 1) simpleGrading")
    t = t.replace("(25 18 18) simpleGrading", "(25 18 1) simpleGrading")
    t = t.replace("(4 5 6 7) (5 10 11 6)", "").replace("(0 3 2 1)", "")
    t = t.replace("(1 2 9 8)", "")
    open(d / "system/blockMeshDict", "w").write(t)
    s = parse(str(d))
    names = [s.patches[p].name for p in range(s.n_patches)]
    assert names[-1] == b"defaultFaces" and s.patches[s.n_patches - 1].type == S.PATCH_EMPTY
    assert s.side_patch[4] == s.side_patch[5] == s.n_patches - 1


def test_missing_file(gpu_lib, tmp_path):
    d = _copy_case(tmp_path)
    os.remove(d / "system/controlDict")
    _expect(d, S.ERR_IO, "controlDict")


def test_obstacle_from_blocks(gpu_lib, tmp_path):
    """Eight blocks around a missing centre column: the hole becomes a solid
    box whose faces carry the patch listed for them."""
    d = _copy_case(tmp_path)
    vid = lambda i, j, k: i + 4 * (j + 4 * k)
    verts = " ".join(f"({i} {j} {k})" for k in range(2) for j in range(4) for i in range(4))
    blocks = []
    for j in range(3):
        for i in range(3):
            if (i, j) == (1, 1):
                continue
            v = [vid(i, j, 0), vid(i + 1, j, 0), vid(i + 1, j + 1, 0), vid(i, j + 1, 0),
                 vid(i, j, 1), vid(i + 1, j, 1), vid(i + 1, j + 1, 1), vid(i, j + 1, 1)]
            blocks.append("hex (" + " ".join(map(str, v)) + ") (2 2 2) simpleGrading (1 1 1)")

    def quad(a, b, c, e):
        return f"({a} {b} {c} {e})"
    faces = {"flow": [], "entrance": [], "walls": []}
    for j in range(3):
        faces["flow"].append(quad(vid(0, j, 0), vid(0, j + 1, 0), vid(0, j + 1, 1), vid(0, j, 1)))
        faces["flow"].append(quad(vid(3, j, 0), vid(3, j + 1, 0), vid(3, j + 1, 1), vid(3, j, 1)))
    for i in range(3):
        faces["flow"].append(quad(vid(i, 0, 0), vid(i + 1, 0, 0), vid(i + 1, 0, 1), vid(i, 0, 1)))
        faces["flow"].append(quad(vid(i, 3, 0), vid(i + 1, 3, 0), vid(i + 1, 3, 1), vid(i, 3, 1)))
    for j in range(3):
        for i in range(3):
            if (i, j) == (1, 1):
                continue
            faces["entrance"].append(quad(vid(i, j, 0), vid(i + 1, j, 0), vid(i + 1, j + 1, 0), vid(i, j + 1, 0)))
            faces["entrance"].append(quad(vid(i, j, 1), vid(i + 1, j, 1), vid(i + 1, j + 1, 1), vid(i, j + 1, 1)))
    faces["walls"] = [quad(vid(1, 1, 0), vid(1, 2, 0), vid(1, 2, 1), vid(1, 1, 1)),
                      quad(vid(2, 1, 0), vid(2, 2, 0), vid(2, 2, 1), vid(2, 1, 1)),
                      quad(vid(1, 1, 0), vid(2, 1, 0), vid(2, 1, 1), vid(1, 1, 1)),
                      quad(vid(1, 2, 0), vid(2, 2, 0), vid(2, 2, 1), vid(1, 2, 1))]
    types = {"flow": "patch", "entrance": "symmetry", "walls": "wall"}
    bnd = "\n".join(f"{n} {{ type {types[n]}; faces ( {' '.join(f)} ); }}" for n, f in faces.items())
    (d / "system/blockMeshDict").write_text(
        "FoamFile { version 2.0; format ascii; class dictionary; object blockMeshDict; }\n"
        f"convertToMeters 0.01;\nvertices ( {verts} );\nblocks ( {' '.join(blocks)} );\n"
        f"boundary ( {bnd} );\n")
    s = parse(str(d))
    assert list(s.n_cells) == [6, 6, 2]
    assert s.n_obstacles == 1
    ob = s.obstacles[0]
    assert list(ob.lo) == [2, 2, 0] and list(ob.hi) == [4, 4, 2]
    assert [ob.patch[q] for q in range(4)] == [2, 2, 2, 2]
