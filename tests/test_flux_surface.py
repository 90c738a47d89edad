"""dsmcFluxSurface (macroscopicProperties/derived/flux/dsmcFluxSurface/
dsmcFluxSurface.C:203-400): the fieldModel that reduces the face tracker's
parcelIdFlux and massIdFlux over a face zone.  Per step it adds, over the
zone's faces and its typeIds, flux x FN x (S/|S| . fluxDirection); at output
time the sums over the averaging time (steps x deltaT) are flow rates and
over the zone's area (sum of |S|) fluxes.

The zone is a topoSet boxToFace box.  The reduction here is restated in
numpy from the face numbering and the mesh geometry; the GPU's values must
equal it on the GPU's own face sums, and a drifting free stream must give
n U through a plane."""
import os
import shutil

import numpy as np
import pytest

from hystrath_gb300 import spec as S

HERE = os.path.dirname(os.path.abspath(__file__))
CORNER = os.path.join(HERE, "golden", "cases", "hypersonic_corner")
COUETTE = os.path.join(HERE, "golden", "cases", "couette_N2-O2")

HEADER = "FoamFile { version 2.0; format ascii; class dictionary; object %s; }\n"


# ------------------------------------------------------------ restatement
def _nodes(spec, a):
    n = spec.n_cells[a]
    if spec.node_coords[a]:
        return np.array([spec.node_coords[a][i] for i in range(n + 1)])
    return spec.origin[a] + spec.cell_size[a] * np.arange(n + 1)


def face_table(spec):
    """Per face of the tracker numbering: axis, centre, area, sign of S along
    the axis and whether it is a mesh face (a fluid cell on one side)."""
    n = [spec.n_cells[a] for a in range(3)]
    nodes = [_nodes(spec, a) for a in range(3)]
    mid = [0.5 * (x[1:] + x[:-1]) for x in nodes]
    wid = [x[1:] - x[:-1] for x in nodes]
    fluid = np.zeros((n[2] + 2, n[1] + 2, n[0] + 2), bool)
    fluid[1:-1, 1:-1, 1:-1] = True
    for o in range(spec.n_obstacles):
        ob = spec.obstacles[o]
        fluid[ob.lo[2] + 1:ob.hi[2] + 1, ob.lo[1] + 1:ob.hi[1] + 1, ob.lo[0] + 1:ob.hi[0] + 1] = False
    cols = {"axis": [], "centre": [], "area": [], "sgn": [], "exists": []}
    for a in range(3):
        dims = [n[2], n[1], n[0]]
        dims[2 - a] += 1                       # (z, y, x) order, x fastest
        k, j, i = np.meshgrid(*[np.arange(d) for d in dims], indexing="ij")
        idx = [i.ravel(), j.ravel(), k.ravel()]
        lo = [q + 1 for q in idx]
        hi = [q + 1 for q in idx]
        lo[a] = idx[a]                          # the cell below plane p is p - 1
        lo_f = fluid[lo[2], lo[1], lo[0]]
        hi_f = fluid[hi[2], hi[1], hi[0]]
        centre = np.empty((len(idx[0]), 3))
        area = np.ones(len(idx[0]))
        for b in range(3):
            if b == a:
                centre[:, b] = nodes[b][idx[b]]
            else:
                centre[:, b] = mid[b][idx[b]]
                area *= wid[b][idx[b]]
        cols["axis"].append(np.full(len(idx[0]), a))
        cols["centre"].append(centre)
        cols["area"].append(area)
        cols["sgn"].append(np.where(lo_f, 1.0, -1.0))
        cols["exists"].append(lo_f | hi_f)
    return {k: np.concatenate(v) for k, v in cols.items()}


def surface_values(spec, flux_of, box_min, box_max, direction, species, steps):
    """faceParticleFlux, faceParticleFlowRate, faceMassFlux, faceMassFlowRate,
    area, averaging time from the face sums (flux_of(name, m))."""
    t = face_table(spec)
    c = t["centre"]
    sel = t["exists"] & np.all(c >= np.asarray(box_min), axis=1) & np.all(c <= np.asarray(box_max), axis=1)
    d = np.asarray(direction, float)
    d = d / np.linalg.norm(d)
    w = spec.n_equivalent_particles * t["sgn"] * d[t["axis"]]
    parcels = sum((flux_of("parcelIdFlux", m) * w)[sel].sum() for m in species)
    mass = sum((flux_of("massIdFlux", m) * w)[sel].sum() for m in species)
    area = t["area"][sel].sum()
    T = steps * spec.delta_t
    return np.array([parcels / T / area, parcels / T, mass / T / area, mass / T, area, T])


def _free_stream_box(n, fn, u, seed):
    """A drifting argon free stream in a box that deletes on every side and
    injects the same stream through every side."""
    s = S.make_box_case(n, 1e-3, S.AR, fn=fn, dt=2e-6, seed=seed, n_density=1e20, t_tra=300.0,
                        velocity=u, side_model=S.BC_DELETION, side_type=S.PATCH_PATCH)
    p = s.patches[0]
    p.inflow = 1
    p.inflow_number_density[0] = 1e20
    p.inflow_t_tra = 300.0
    for a in range(3):
        p.inflow_velocity[a] = u[a]
    return s


# ------------------------------------------------------------ case files
def _flux_case(tmp_path, src=CORNER, zone_form="faceZoneSet", type_ids="(Ar)",
               box="(0.1 -1 -1) (0.1001 1 1)", direction="(2 0 0)", zone="plane"):
    d = tmp_path / "case"
    shutil.copytree(src, d)
    fp = d / "system" / "fieldPropertiesDict"
    text = fp.read_text()
    entry = ("    surface\n    {\n        fieldModel dsmcFluxSurface;\n"
             "        timeProperties { timeOption write; resetAtOutput on; }\n"
             "        dsmcFluxSurfaceProperties { fieldName Ar; faceZoneName %s; typeIds %s;"
             " fluxDirection %s; }\n    }\n" % (zone, type_ids, direction))
    i = text.rindex(");")
    fp.write_text(text[:i] + entry + text[i:])
    if zone_form == "faceZoneSet":
        actions = ("    { name planeSet; type faceSet; action new; source boxToFace;"
                   " sourceInfo { box %s; } }\n"
                   "    { name plane; type faceZoneSet; action new; source setToFaceZone;"
                   " sourceInfo { faceSet planeSet; } }\n" % box)
    else:   # a faceSet that setsToZones turns into a zone of the same name
        actions = "    { name plane; type faceSet; action new; source boxToFace; box %s; }\n" % box
    (d / "system" / "topoSetDict").write_text(HEADER % "topoSetDict" + "actions\n(\n" + actions + ");\n")
    return str(d)


@pytest.mark.parametrize("form", ["faceZoneSet", "faceSet"])
def test_parse_flux_surfaces(gpu_lib, tmp_path, form):
    from hystrath_gb300.dsmc import parse_flux_surfaces
    d = _flux_case(tmp_path, zone_form=form)
    (f,) = parse_flux_surfaces(d)
    assert f.zone_name == b"plane" and f.field_name == b"Ar"
    assert list(f.box_min) == [0.1, -1, -1] and list(f.box_max) == [0.1001, 1, 1]
    assert list(f.direction) == [2, 0, 0] and f.species_mask == 1
    assert parse_flux_surfaces(CORNER) == []


@pytest.mark.parametrize("bad,msg", [({"type_ids": "(N2)"}, "Cannot find typeId: N2"),
                                     ({"zone": "nowhere"}, "Cannot find region: nowhere")])
def test_parse_flux_surface_errors(gpu_lib, tmp_path, bad, msg):
    from hystrath_gb300.dsmc import DsmcError, parse_flux_surfaces
    d = _flux_case(tmp_path, **bad)
    with pytest.raises(DsmcError) as e:
        parse_flux_surfaces(d)
    assert msg in str(e.value) and e.value.code == 4


def test_restated_geometry():
    """The restatement's faces: counts per axis, no face inside the solid
    cube, outward signs on the low sides of the domain and of the cube."""
    s = S.config2(seed=1, scale=8)
    t = face_table(s)
    n = [s.n_cells[a] for a in range(3)]
    assert len(t["axis"]) == (n[0] + 1) * n[1] * n[2] + n[0] * (n[1] + 1) * n[2] + n[0] * n[1] * (n[2] + 1)
    ob = s.obstacles[0]
    e = [ob.hi[a] - ob.lo[a] for a in range(3)]
    inside = sum((e[a] - 1) * e[(a + 1) % 3] * e[(a + 2) % 3] for a in range(3))
    assert inside > 0 and (~t["exists"]).sum() == inside
    x = t["centre"][:, 0]
    assert np.all(t["sgn"][t["exists"] & (t["axis"] == 0) & (x == s.origin[0])] == -1.0)
    # the cube's +x side: faces whose low cell is solid, high cell fluid
    xc = s.origin[0] + ob.hi[0] * s.cell_size[0]
    on = t["exists"] & (t["axis"] == 0) & np.isclose(x, xc, rtol=0, atol=1e-12)
    y, z = t["centre"][:, 1], t["centre"][:, 2]
    cube = on & (y > s.origin[1] + ob.lo[1] * s.cell_size[1]) & (y < s.origin[1] + ob.hi[1] * s.cell_size[1]) \
        & (z > s.origin[2] + ob.lo[2] * s.cell_size[2]) & (z < s.origin[2] + ob.hi[2] * s.cell_size[2])
    assert cube.sum() == e[1] * e[2] and np.all(t["sgn"][cube] == -1.0) and np.all(t["sgn"][on & ~cube] == 1.0)


def _plane_values(flux_of, spec, axis, planes, direction, steps):
    """One zone per node plane of the axis (a box thin enough to hold only
    that plane's faces)."""
    h = spec.cell_size[axis]
    out = []
    for p in planes:
        lo, hi = [-1.0] * 3, [1.0] * 3
        lo[axis], hi[axis] = p * h - 1e-3 * h, p * h + 1e-3 * h
        out.append(surface_values(spec, flux_of, lo, hi, direction, [0], steps))
    return np.array(out)


def test_oracle_free_stream_flux(oracle_mod):
    """n U_x through the internal x planes of a drifting free stream (5%,
    about 4 standard deviations of the plane mean); the mass flux is m times
    the number flux; a reversed direction flips the signs."""
    n, u = (8, 8, 8), (1000.0, 150.0, -80.0)
    s = _free_stream_box(n, 4e8, u, seed=3)
    o = oracle_mod.OracleCloud(s, threads=4)
    o.initialise()
    o.set_face_tracking(True)
    steps = 80
    for _ in range(steps):
        o.run_phases(S.PHASE_INFLOW | S.PHASE_MOVE | S.PHASE_SORT)
    v = _plane_values(o.face_flux, s, 0, range(1, 8), (1, 0, 0), steps)
    np.testing.assert_allclose(v[:, 4], 64e-6, rtol=1e-12)
    np.testing.assert_allclose(v[:, 5], steps * s.delta_t, rtol=1e-15)
    assert v[:, 0].mean() == pytest.approx(1e20 * u[0], rel=0.05)
    np.testing.assert_allclose(v[:, 2], v[:, 0] * S.AR["mass"], rtol=1e-9)
    r = _plane_values(o.face_flux, s, 0, range(1, 8), (-3, 0, 0), steps)
    np.testing.assert_allclose(r[:, :4], -v[:, :4], rtol=1e-12)


# ------------------------------------------------------------ GPU
@pytest.mark.gpu
@pytest.mark.parametrize("case", ["channel_cube", "couette", "corner"])
def test_gpu_flux_surfaces_equal_the_face_reduction(gpu_lib, case):
    """Several zones (an internal plane, a domain side, the faces around the
    solid cube, a slanted direction, one species of two) on the GPU's own
    face sums: equal to the restated reduction."""
    from hystrath_gb300.dsmc import DsmcCloud, parse_case
    spec = {"channel_cube": lambda: S.config2(seed=7, scale=8),
            "couette": lambda: parse_case(COUETTE),
            "corner": lambda: parse_case(CORNER)}[case]()
    g = DsmcCloud(spec)
    g.initialise()
    lo = np.array([spec.origin[a] if not spec.node_coords[a] else spec.node_coords[a][0] for a in range(3)])
    hi = np.array([_nodes(spec, a)[-1] for a in range(3)])
    ext = hi - lo
    zones = [("mid_x", lo + [0.49 * ext[0], -1, -1], lo + [0.51 * ext[0], 2 * ext[1], 2 * ext[2]], (1, 0, 0)),
             ("side", lo - 1, lo + [1e-12, 2 * ext[1], 2 * ext[2]], (-1, 0, 0)),
             ("all", lo - 1, hi + 1, (0.3, -0.5, 0.8))]
    sp_sets = [None, [spec.n_species - 1], None]
    for (name, a, b, d), sp in zip(zones, sp_sets):
        g.add_flux_surface(name, a, b, d, species=sp)
    g.evolve(6)
    assert g.n_flux_surfaces() == 3
    for i, ((name, a, b, d), sp) in enumerate(zip(zones, sp_sets)):
        got = g.flux_surface(i)
        assert got["zone_name"] == name
        want = surface_values(spec, g.face_flux, a, b, d, range(spec.n_species) if sp is None else sp, 6)
        np.testing.assert_allclose([got[k] for k in S.FLUX_SURFACE_VALUES], want, rtol=1e-12, atol=1e-300)
    # the time window restarts with the sampling
    g.reset_sampling()
    from hystrath_gb300.dsmc import DsmcError
    with pytest.raises(DsmcError):
        g.flux_surface(0)
    g.evolve(2)
    assert g.flux_surface(0)["averaging_time"] == pytest.approx(2 * spec.delta_t, rel=1e-15)


@pytest.mark.gpu
def test_gpu_free_stream_flux(gpu_lib):
    """n U through internal planes of a drifting free stream (x: 1.5%, y:
    10%, each about 4 standard deviations of the plane mean), on the GPU's
    surfaces."""
    from hystrath_gb300.dsmc import DsmcCloud
    u = (1000.0, 150.0, -80.0)
    s = _free_stream_box((24, 24, 24), 4e8, u, seed=5)
    g = DsmcCloud(s)
    g.initialise()
    h = s.cell_size[0]
    for axis in (0, 1):
        for p in range(1, 24):
            lo, hi = [-1.0] * 3, [1.0] * 3
            lo[axis], hi[axis] = p * h - 1e-3 * h, p * h + 1e-3 * h
            d = [0, 0, 0]
            d[axis] = 1
            g.add_flux_surface(f"{'xy'[axis]}{p}", lo, hi, d)
    g.evolve(100)
    v = [g.flux_surface(i) for i in range(g.n_flux_surfaces())]
    for x in v:
        assert x["area"] == pytest.approx(576e-6, rel=1e-12)
        assert x["faceMassFlux"] == pytest.approx(x["faceParticleFlux"] * S.AR["mass"], rel=1e-9)
    assert np.mean([x["faceParticleFlux"] for x in v[:23]]) == pytest.approx(1e20 * u[0], rel=0.015)
    assert np.mean([x["faceParticleFlux"] for x in v[23:]]) == pytest.approx(1e20 * u[1], rel=0.1)


@pytest.mark.gpu
def test_gpu_case_directory_flux_surface(gpu_lib, tmp_path):
    """dsmc_create reads the surface from fieldPropertiesDict and topoSetDict;
    every output time appends one line to each of the four .xy files."""
    from hystrath_gb300.dsmc import DsmcCloud, parse_case
    d = _flux_case(tmp_path)
    g = DsmcCloud(d)
    assert g.n_flux_surfaces() == 1
    g.initialise()
    g.evolve(5)
    v1 = g.flux_surface(0)
    spec = parse_case(d)
    want = surface_values(spec, g.face_flux, (0.1, -1, -1), (0.1001, 1, 1), (2, 0, 0), [0], 5)
    np.testing.assert_allclose([v1[k] for k in S.FLUX_SURFACE_VALUES], want, rtol=1e-12, atol=1e-300)
    assert v1["area"] == pytest.approx(0.18 * 0.18, rel=1e-12)
    g.write_flux_surfaces(d, 5 * spec.delta_t)
    g.evolve(5)
    g.write_flux_surfaces(d, 10 * spec.delta_t)
    for k in ("faceParticleFlux", "faceParticleFlowRate", "faceMassFlux", "faceMassFlowRate"):
        rows = np.loadtxt(os.path.join(d, "fieldMeasurements", f"{k}_plane_Ar.xy"))
        assert rows.shape == (2, 2)
        assert rows[0, 1] == pytest.approx(v1[k], rel=1e-10)
        assert rows[1, 0] == pytest.approx(10 * spec.delta_t, rel=1e-10)


@pytest.mark.gpu
def test_gpu_case_with_an_empty_zone_is_rejected(gpu_lib, tmp_path):
    """A zone whose box holds no face centre fails dsmc_create with the
    reference's message, and the half-made cloud is released."""
    from hystrath_gb300.dsmc import DsmcCloud, DsmcError
    d = _flux_case(tmp_path, box="(0.1003 -1 -1) (0.1004 1 1)")
    with pytest.raises(DsmcError) as e:
        DsmcCloud(d)
    assert "Cannot find region: plane" in str(e.value) and e.value.code == 4
    g = DsmcCloud(CORNER)   # the library stays usable
    assert g.n_flux_surfaces() == 0
    g.close()
