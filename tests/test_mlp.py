"""The learned (sigma_T c_R)max: the oracle's gradient formulas against finite
differences (CPU), the GPU kernels against the oracle (forward, gradient),
training, and what the trained network gains inside noTimeCounter (GPU)."""
import numpy as np
import pytest

from hystrath_gb300 import spec as S
from oracle import mlp_oracle as MO


def _data(n, seed=0):
    rng = np.random.default_rng(seed)
    X = np.stack([rng.uniform(40.0, 48.0, n), rng.uniform(5.0, 10.0, n), rng.uniform(0.0, 12.0, n)], 1)
    # a smooth target in the range of log (sigma_T c_R)max
    Y = -40.0 + 0.26 * X[:, 1] + 0.05 * np.sin(X[:, 2]) + 0.01 * (X[:, 0] - 44.0) ** 2
    return X.astype(np.float32), Y.astype(np.float32)


def _norm(X, Y):
    from hystrath_gb300.learn import fit_norm
    return fit_norm(X, Y)


def _params(seed=0):
    from hystrath_gb300.learn import init_params
    return init_params(seed)


def test_bf16_rounding():
    v = np.array([1.0, 1.0 + 2 ** -9, 1.0 + 3 * 2 ** -9, -2.5, 3.14159265], dtype=np.float32)
    r = MO.bf16(v)
    assert r[0] == 1.0
    assert r[1] == 1.0                     # halfway: ties to even
    assert r[2] == np.float32(1.0 + 2 ** -7)
    assert r[3] == -2.5
    assert abs(r[4] - 3.140625) < 1e-7


def test_oracle_gradient_matches_finite_differences():
    X, Y = _data(64, 1)
    nm = _norm(X, Y)
    p = _params(3).astype(np.float64)
    loss, g = MO.loss_grad(p, nm, X, Y, exact=True)
    rng = np.random.default_rng(0)
    idx = np.concatenate([rng.choice(np.arange(MO.OFF_W1, MO.OFF_B1), 6, replace=False),
                          rng.choice(np.arange(MO.OFF_W2, MO.OFF_B2), 10, replace=False),
                          [MO.OFF_B1 + 5, MO.OFF_B2 + 7, MO.OFF_W3 + 9, MO.OFF_B3]])
    h = 1e-6
    for i in idx:
        pp = p.copy(); pp[i] += h
        pm = p.copy(); pm[i] -= h
        fd = (MO.loss_grad(pp, nm, X, Y, exact=True)[0] - MO.loss_grad(pm, nm, X, Y, exact=True)[0]) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(g[i])) + 1e-8, (i, fd, g[i])


def test_learn_module_needs_no_gpu_to_import():
    from hystrath_gb300 import learn
    p = learn.init_params(0)
    assert p.shape == (MO.NPARAM,) and np.all(np.abs(p[MO.OFF_W2:MO.OFF_B2]) <= 0.125 + 1e-7)


@pytest.mark.gpu
def test_gpu_forward_matches_oracle():
    from hystrath_gb300.dsmc import Mlp
    X, Y = _data(1000, 2)
    nm = _norm(X, Y)
    p = _params(1)
    m = Mlp()
    m.set_params(p, nm)
    got = m.predict(X)
    want = MO.predict(p, nm, X)
    # same bf16 roundings; FP32 sums in a different order can move a rounding
    # by one bf16 step
    assert np.max(np.abs(got - want)) < 2e-2 * nm[7]
    assert np.mean(np.abs(got - want)) < 2e-3 * nm[7]


@pytest.mark.gpu
@pytest.mark.parametrize("n", [64, 1000, 4099])
def test_gpu_gradient_matches_oracle(n):
    from hystrath_gb300.dsmc import Mlp
    X, Y = _data(n, 5)
    nm = _norm(X, Y)
    p = _params(2)
    m = Mlp()
    m.set_params(p, nm)
    g, loss = m.grad(X, Y)
    lo, go = MO.loss_grad(p, nm, X, Y)
    assert abs(loss - lo) <= 1e-3 * lo
    rel = np.linalg.norm(g - go) / np.linalg.norm(go)
    assert rel < 1e-2, rel
    # every parameter block carries its own gradient
    for a, b in ((MO.OFF_W1, MO.OFF_B1), (MO.OFF_B1, MO.OFF_W2), (MO.OFF_W2, MO.OFF_B2),
                 (MO.OFF_B2, MO.OFF_W3), (MO.OFF_W3, MO.OFF_B3)):
        assert np.linalg.norm(g[a:b] - go[a:b]) <= 2e-2 * np.linalg.norm(go[a:b]) + 1e-9


@pytest.mark.gpu
def test_gpu_training_fits_and_is_reproducible():
    from hystrath_gb300.dsmc import Mlp
    from hystrath_gb300.learn import init_params
    X, Y = _data(200_000, 7)
    nm = _norm(X, Y)
    losses = []
    params = []
    for _ in range(2):
        m = Mlp()
        m.set_params(init_params(0), nm)
        m.set_data(X, Y)
        loss = m.train(600, 4096, 1e-3, seed=5)
        losses.append(loss)
        params.append(m.params()[0])
    assert np.mean(losses[0][-50:]) < 0.05 * np.mean(losses[0][:10])
    assert np.array_equal(params[0], params[1])            # no atomics in the reduction
    assert np.array_equal(losses[0], losses[1])


@pytest.mark.gpu
def test_learned_selection_draws_fewer_candidates_at_the_same_rate():
    """A network trained on a plain heat bath's recorded maxima: the learned
    run of the same heat bath draws fewer candidates per accepted collision and
    keeps the collision count of the plain run."""
    from hystrath_gb300 import learn
    from hystrath_gb300 import spec as S
    from hystrath_gb300.dsmc import DsmcCloud

    def make(seed):
        return S.config1(seed=seed, n=24)

    X, Y = learn.collect(make, [0, 1], [5, 20, 40, 80, 160])
    # the 0.95-quantile of the recorded maxima given the cell state
    model, loss = learn.train(X, Y, steps=1500, batch=8192, seed=0, tau=0.95)
    margin = 0.0
    steps = 300

    def run(learned):
        g = DsmcCloud(make(9))
        g.initialise()
        g.evolve(100)
        if learned:
            g.set_learned(model, 10, margin)
        g.set_selection_audit(True)
        i0 = g.info()
        g.evolve(steps)
        i1 = g.info()
        audit = learn.audit_summary(g.cell_array("selectionAudit"))
        g.close()
        return i1.collisions_total - i0.collisions_total, i1.candidates_total - i0.candidates_total, audit

    cp, kp, ap = run(False)
    cl, kl, al = run(True)
    # fewer candidates per accepted collision (a cell whose prediction was
    # exceeded stays on the running maximum until a prediction covers the
    # product, which keeps the saving small)
    assert kl / cl < 0.995 * (kp / cp), (kp / cp, kl / cl)
    # both are counts of about 1e6: 1% is several standard errors
    assert abs(cl / cp - 1) < 0.01, (cp, cl)
    # the audit: the expected per-cell shortfall of the collision count that
    # a maximum below the product causes -- tiny for the running maximum,
    # within 1% in total and in almost every cell for the learned one
    assert ap["expected_shortfall_total"] < 1e-3, ap
    assert al["expected_shortfall_total"] < 0.005, al
    assert al["cells_above_1pct"] < ap["cells_above_1pct"] + 0.05, (al, ap)


def _features_restated(g):
    """The learned maximum's inputs restated from the cloud's parcels: the
    same exact fixed-point sums per cell (mass weight round(256 m/m0),
    velocity round(16 u)), then the features in FP32."""
    st = g.particles()
    sp = g.spec
    m0 = sp.species[0].mass
    mrel = np.array([np.float32(sp.species[q].mass / m0) for q in range(sp.n_species)], dtype=np.float32)
    w = np.rint(mrel * np.float32(256.0)).astype(np.int64)[st["species"]]
    u = np.rint(st["U"] * 16.0).astype(np.int64)
    c = st["cell"].astype(np.int64)
    C = g.n_cells
    N = np.bincount(c, minlength=C).astype(np.int64)
    W = np.bincount(c, weights=w, minlength=C).astype(np.int64)      # exact below 2^53
    WU = [np.zeros(C, np.int64) for _ in range(3)]
    for a in range(3):
        np.add.at(WU[a], c, w * u[:, a])
    WUU = np.zeros(C, np.int64)
    np.add.at(WUU, c, w * (u * u).sum(1))
    f32 = np.float32
    M = W.astype(f32) * f32(1 / 256)
    Mu = [x.astype(f32) * f32(1 / 4096) for x in WU]
    Muu = WUU.astype(f32) * f32(1 / 65536)
    with np.errstate(divide="ignore", invalid="ignore"):
        U2 = (Mu[0] * Mu[0] + Mu[1] * Mu[1] + Mu[2] * Mu[2]) / (M * M)
        kOverM0 = f32(1.380649e-23 / m0)
        T = (Muu - M * U2) / (f32(3.0) * kOverM0 * N.astype(f32))
        nd = f32(sp.n_equivalent_particles / np.prod([sp.cell_size[a] for a in range(3)]))
        cmp = np.sqrt(f32(2.0) * kOverM0 * T / (M / N.astype(f32)))
        valid = (N >= 2) & (T > 0)
        out = np.zeros((C, 4), np.float32)
        out[valid, 0] = np.log(nd * N[valid].astype(f32))
        out[valid, 1] = np.log(T[valid])
        out[valid, 2] = np.sqrt(U2[valid]) / cmp[valid]
        out[valid, 3] = 1.0
    return out


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["channel", "mixture"])
def test_cell_features_match_a_restatement(gpu_lib, case):
    """The feature pass (warp runs of equal cells summed before the shared
    sums) against a numpy restatement of the same exact sums: the developed
    channel at 1/8 scale (one species, two or three cells per warp) and an
    N2-Ar box (mass weights 256 and 365)."""
    from hystrath_gb300.dsmc import DsmcCloud
    if case == "channel":
        s = S.config2(seed=31, scale=8)
    else:
        s = S.make_box_case((12, 12, 12), 1e-3, S.N2, fn=2e9, dt=2e-7, seed=32, n_density=5e19,
                            t_tra=3000.0, t_rot=300.0, t_vib=300.0, side_model=S.BC_SPECULAR,
                            collision=S.COLL_LB_VHS)
        s.n_species = 2
        S.set_species(s, 1, S.AR)
        s.init_number_density[1] = 5e19
    g = DsmcCloud(s)
    g.initialise()
    g.evolve(60)
    got = g.cell_array("learnedFeatures")
    want = _features_restated(g)
    g.close()
    assert np.array_equal(got[:, 3], want[:, 3])
    v = want[:, 3] == 1
    assert v.sum() > 0.5 * len(v)
    np.testing.assert_allclose(got[v, 0], want[v, 0], rtol=3e-7, atol=0)     # log n: exact counts, logf ulps
    np.testing.assert_allclose(got[v, 1], want[v, 1], rtol=0, atol=1e-4)      # log T: FP32 cancellation
    np.testing.assert_allclose(got[v, 2], want[v, 2], rtol=1e-4, atol=1e-6)
