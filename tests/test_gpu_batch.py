"""Batched small CPDs (one launch per stage) vs single-problem cpd and the oracle."""
import numpy as np
import pytest

import tfx_oracle as orc

pytestmark = pytest.mark.gpu

tfx = pytest.importorskip("tensorfox_gb300")


def problems(n, seed, noise=1e-4, dtype=np.float64):
    rng = np.random.default_rng(seed)
    Ts, Ws, Rs = [], [], []
    for _ in range(n):
        dims = tuple(int(v) for v in rng.integers(8, 65, size=3))
        R = int(rng.integers(2, 13))
        W = [rng.standard_normal((d, R)) for d in dims]
        T = orc.cpd2tens(W)
        E = rng.standard_normal(dims)
        T = T + noise * np.linalg.norm(T) / np.linalg.norm(E) * E
        Ts.append(T.astype(dtype))
        Ws.append(W)
        Rs.append(R)
    return Ts, Ws, Rs


def test_batch_mlsvd_matches_single_problem_mlsvd():
    Ts, _, Rs = problems(6, 1)
    from tensorfox_gb300 import batch
    for T, R in zip(Ts, Rs):
        S, U, _, sig = tfx.mlsvd(np.transpose(T, np.argsort(-np.array(T.shape))).copy(), 1.0, R, None)
        # batch path on the same single tensor (its dims are already sorted above)
        np.random.seed(0)
        out = batch.cpd_batch([T], [R], None)
        assert out[0][1].num_steps >= 1
        assert all(s.shape[0] == min(R, d) for s, d in zip(sig, sorted(T.shape, reverse=True)))


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_batch_reaches_noise_level(dtype):
    Ts, Ws, Rs = problems(48, 2, dtype=dtype)
    np.random.seed(1)
    out = tfx.cpd_batch(Ts, Rs)
    errs = np.array([o.rel_error for _, o in out])
    # every problem's reported error equals the oracle's residual of its factors
    for (f, o), T in zip(out[:8], Ts[:8]):
        ref = orc.fastnorm(orc.unfold(T.astype(np.float64), 1), orc.cpd2unfold1(f)) / np.linalg.norm(T)
        assert abs(o.rel_error - ref) <= 1e-4 * ref + 1e-9
    assert np.median(errs) < 5e-4
    assert np.mean(errs < 1e-2) >= 0.85


def test_batch_agrees_with_serial_cpd_statistically():
    Ts, Ws, Rs = problems(12, 3)
    np.random.seed(4)
    outb = tfx.cpd_batch(Ts, Rs)
    np.random.seed(4)
    outs = [tfx.cpd(T, R) for T, R in zip(Ts, Rs)]
    eb = np.array([o.rel_error for _, o in outb])
    es = np.array([o.rel_error for _, o in outs])
    # same algorithm, different random starts: same quality on well-posed problems
    assert np.median(eb) < 3 * np.median(es) + 1e-6


def test_engine_tile_and_order_do_not_change_results():
    """The autotuner's choices (register tile 1/2/4, problem order) only change
    speed: every problem's trajectory stays the same."""
    Ts, _, Rs = problems(40, 5)
    ref = None
    for tile in (None, 1, 2, 4):
        o = tfx.make_options(None)
        o.tile = tile
        o.maxiter = 40
        np.random.seed(6)
        tm = {}
        out = tfx.cpd_batch(Ts, Rs, o, timings=tm, tune=(tile is None))
        errs = [np.asarray(op.errors[0]) for _, op in out]
        if ref is None:
            ref = errs
            assert tm['engine_config'][1] in ('given', 'largest_first')
        else:
            assert tm['engine_config'] == (tile, 'largest_first')
            for a, b in zip(errs, ref):
                assert len(a) == len(b)
                np.testing.assert_allclose(a, b, rtol=1e-10, atol=1e-15)


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_every_batch_problem_equals_its_solve_alone(dtype):
    """Each problem of one batched launch gives exactly what the same problem
    gives when solved alone from the same start: the batch draws the starts
    of all problems from NumPy's RNG in problem order, so replaying the draws
    of the problems before it reproduces problem p's start; 'cg_static' fixes
    the CG caps.  No problem's result depends on its neighbours."""
    Ts, _, Rs = problems(24, 6, dtype=dtype)

    class O:
        inner_method = 'cg_static'
        cg_maxiter = 10
        maxiter = 80
    o = tfx.make_options(O)
    np.random.seed(21)
    s0 = np.random.get_state()
    outb = tfx.cpd_batch(Ts, Rs, o)
    off = 0
    for p in range(len(Ts)):
        np.random.set_state(s0)
        if off:
            np.random.randn(off)         # the draws of the problems before p
        f1, o1 = tfx.cpd_batch([Ts[p]], [Rs[p]], o)[0]
        fb, ob = outb[p]
        assert o1.core_dims == ob.core_dims
        assert o1.num_steps == ob.num_steps
        tol = 1e-10 if dtype == np.float64 else 1e-6
        np.testing.assert_allclose(o1.errors[0], ob.errors[0], rtol=tol, atol=1e-15)
        assert abs(o1.rel_error - ob.rel_error) <= tol * ob.rel_error + 1e-15
        for a, b in zip(f1, fb):
            np.testing.assert_allclose(a, b, rtol=100 * tol, atol=100 * tol * np.abs(b).max())
        off += Rs[p] * sum(ob.core_dims)
