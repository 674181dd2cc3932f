"""Pins the CPU oracle against fixtures produced by the reference itself."""
import numpy as np
import pytest

import tfx_oracle as orc
from conftest import load_golden, split_x

UNIT_CASES = ["units_L3", "units_L4", "units_L3_big", "units_L5"]


@pytest.mark.parametrize("name", UNIT_CASES)
def test_units_match_reference(name):
    g = load_golden(name)
    dims, R = [int(d) for d in g["dims"]], int(g["R"])
    W = split_x(g["x"], dims, R)
    Gr, P1, P2 = orc.gramians(W)
    np.testing.assert_allclose(Gr, g["Gr"], rtol=1e-13, atol=1e-13)
    np.testing.assert_allclose(P1, g["P1"], rtol=1e-13, atol=1e-12)
    L = len(dims)
    for l in range(L):
        for k in range(L):
            if l != k:
                np.testing.assert_allclose(P2[l, k], g["P2"][l, k], rtol=1e-13, atol=1e-12)
    Gamma, gamma = orc.regularization(P1, dims, R)
    np.testing.assert_allclose(Gamma, g["Gamma"], rtol=1e-13)
    M = orc.precond(Gamma, gamma, float(g["damp"]), dims)
    np.testing.assert_allclose(M, g["M"], rtol=1e-13)
    T = g["T"]
    Tl = [orc.unfold(T, l + 1) for l in range(L)]
    np.testing.assert_allclose(orc.compute_grad(Tl, W, P1), g["grad"], rtol=1e-11, atol=1e-11)
    np.testing.assert_allclose(orc.matvec(W, P1, P2, g["v"]), g["matvec"], rtol=1e-11, atol=1e-11)
    y, cgrad, jtj, itn, rn = orc.cg(Tl, [w.copy() for w in W], float(g["damp"]), int(g["cg_iters"]), 0.0)
    np.testing.assert_allclose(cgrad, g["cg_grad"], rtol=1e-11, atol=1e-11)
    np.testing.assert_allclose(jtj, g["cg_jtj"], rtol=1e-10, atol=1e-10)
    np.testing.assert_allclose(y, g["cg_y"], rtol=1e-8, atol=1e-10)
    assert itn == int(g["cg_itn"])
    np.testing.assert_allclose(rn, g["cg_rn"], rtol=1e-6, atol=1e-14)
    np.testing.assert_allclose(orc.cpd2unfold1(W), g["T1_approx"], rtol=1e-12, atol=1e-12)
    assert abs(orc.fastnorm(Tl[0], g["T1_approx"]) - float(g["fastnorm"])) < 1e-10 * float(g["fastnorm"])
    eq = orc.x2cpd(g["x"] * 1.5, [w.copy() for w in W])
    np.testing.assert_allclose(orc.cpd2flat(eq), g["eq_x"], rtol=1e-13)


def test_khatri_rao_and_unfold():
    g = load_golden("kr_unfold")
    np.testing.assert_allclose(orc.khatri_rao(g["A"], g["B"]), g["KR"], rtol=0, atol=0)
    T = g["T"]
    flat = np.concatenate([orc.unfold(T, m + 1).flatten() for m in range(4)])
    np.testing.assert_array_equal(flat, g["unf"])
    for m in range(4):
        np.testing.assert_array_equal(orc.foldback(orc.unfold(T, m + 1), m + 1, T.shape), T)


def _opts(g):
    o = orc.Options()
    for k, v in zip(g["opt_names"], g["opt_values"]):
        setattr(o, str(k), eval(str(v)))
    return orc.make_options(o)


@pytest.mark.parametrize("name", ["dgn_static_L3", "dgn_cg_L3", "dgn_cg_L4", "dgn_small_L3"])
def test_dgn_trajectory_matches_reference(name):
    g = load_golden(name)
    dims, R = [int(d) for d in g["dims"]], int(g["R"])
    o = _opts(g)
    np.random.seed(int(g["seed"]))
    bf, ss, er, im, gr, st = orc.dGN(g["T"], split_x(g["init_x"], dims, R), R, o)
    assert st == int(g["stop"])
    assert len(er) == len(g["errors"])
    np.testing.assert_allclose(er, g["errors"], rtol=1e-6, atol=1e-12)
    np.testing.assert_allclose(ss, g["step_sizes"], rtol=1e-5, atol=1e-12)
    np.testing.assert_allclose(orc.cpd2flat(bf), g["best_x"], rtol=1e-5, atol=1e-8)


INNER_CASES = ["dgn_als_L3", "dgn_als_L4", "dgn_als_fix_L3", "dgn_direct_L3", "dgn_direct_L4", "dgn_direct_fix_L3",
               "dgn_direct_symm_L3", "dgn_direct_big_L3", "dgn_mixed_L3", "dgn_symm_direct_alias_L3",
               "dgn_fix_cg_L3", "dgn_fix_cgr_L3"]
SYMM_CASES = ["dgn_symm_L3", "dgn_symm_alias_L3", "dgn_symm_norm_L3"]
OPTION_CASES = ["dgn_damp_sched_L3", "dgn_norm_L3"]


def start_of(g):
    """The starting factors of a golden dGN case, the fixed one wrapped as [W]."""
    dims, R = [int(d) for d in g["dims"]], int(g["R"])
    f = split_x(g["init_x"], dims, R)
    if int(g.get("alias", 0)):
        return [f[0]] * len(dims)     # one array for every mode
    fix = int(g.get("fix", -1))
    if fix >= 0:
        f[fix] = [f[fix]]
    return f


@pytest.mark.parametrize("name", INNER_CASES)
def test_dgn_inner_als_direct_match_reference(name):
    """dGN with the 'als' and 'direct' inner methods (GaussNewton.py:275-281,
    630-653), fixed factors included, against the reference's trajectories."""
    g = load_golden(name)
    R = int(g["R"])
    o = _opts(g)
    np.random.seed(int(g["seed"]))      # the 'cg' caps draw from the global RNG
    bf, ss, er, im, gr, st = orc.dGN(g["T"], start_of(g), R, o)
    assert st == int(g["stop"])
    assert len(er) == len(g["errors"])
    np.testing.assert_allclose(er, g["errors"], rtol=1e-7, atol=1e-13)
    np.testing.assert_allclose(ss, g["step_sizes"], rtol=1e-6, atol=1e-13)
    np.testing.assert_allclose(gr, g["gradients"], rtol=1e-6, atol=1e-12)   # NaN for 'als' steps
    np.testing.assert_allclose(orc.cpd2flat(bf), g["best_x"], rtol=1e-6, atol=1e-9)


@pytest.mark.parametrize("name", OPTION_CASES)
def test_dgn_options_match_reference(name):
    """A damping schedule (``init_damp`` as a list, GaussNewton.py:110-111,
    490-495) and ``factors_norm`` (Conversion.py:439-442) on the CG path."""
    g = load_golden(name)
    R = int(g["R"])
    np.random.seed(int(g["seed"]))
    bf, ss, er, im, gr, st = orc.dGN(g["T"], start_of(g), R, _opts(g))
    assert st == int(g["stop"])
    assert len(er) == len(g["errors"])
    np.testing.assert_allclose(er, g["errors"], rtol=1e-7, atol=1e-13)
    np.testing.assert_allclose(ss, g["step_sizes"], rtol=1e-6, atol=1e-13)
    np.testing.assert_allclose(orc.cpd2flat(bf), g["best_x"], rtol=1e-6, atol=1e-9)


@pytest.mark.parametrize("name", SYMM_CASES)
def test_dgn_symm_matches_reference(name):
    """symm=True with the CG inner method: the reference's in-place transform
    on a list that holds one array L times (a symmetric start, or any
    iteration after the first) is part of the trajectory."""
    g = load_golden(name)
    R = int(g["R"])
    np.random.seed(int(g["seed"]))
    bf, ss, er, im, gr, st = orc.dGN(g["T"], start_of(g), R, _opts(g))
    assert st == int(g["stop"])
    assert len(er) == len(g["errors"])
    np.testing.assert_allclose(er, g["errors"], rtol=1e-7, atol=1e-13)
    np.testing.assert_allclose(ss, g["step_sizes"], rtol=1e-6, atol=1e-13)


def test_hessian_is_jtj():
    """``hessian`` equals J^T J of the CP map, J formed by finite differences."""
    rng = np.random.default_rng(3)
    dims, R = (4, 3, 5), 2
    W = [rng.standard_normal((d, R)) for d in dims]
    _, P1, P2 = orc.gramians(W)
    H = orc.hessian(W, P1, P2, exact=True)
    x = orc.cpd2flat(W)
    n = len(x)
    J = np.empty((int(np.prod(dims)), n))
    for k in range(n):
        e = np.zeros(n)
        e[k] = 1.0
        fp = orc.cpd2tens(split_x(x + 1e-6 * e, dims, R)).ravel()
        fm = orc.cpd2tens(split_x(x - 1e-6 * e, dims, R)).ravel()
        J[:, k] = (fp - fm) / 2e-6
    np.testing.assert_allclose(H, J.T @ J, rtol=1e-6, atol=1e-6)


def test_hessian_truncation_rule():
    """The reference's blocks (l, m), l > m, keep only their leading R d_l
    columns; with equal dimensions nothing is truncated."""
    rng = np.random.default_rng(4)
    R = 2
    for dims in [(5, 4, 3), (4, 4, 4), (4, 3, 3, 2)]:
        W = [rng.standard_normal((d, R)) for d in dims]
        _, P1, P2 = orc.gramians(W)
        H, J = orc.hessian(W, P1, P2), orc.hessian(W, P1, P2, exact=True)
        sd = orc.sum_dims_of(dims, R)
        want = J.copy()
        for l in range(len(dims)):
            for m in range(l):
                want[sd[l]:sd[l + 1], sd[m] + R * dims[l]:sd[m + 1]] = 0.0
                want[sd[m] + R * dims[l]:sd[m + 1], sd[l]:sd[l + 1]] = 0.0
        np.testing.assert_array_equal(H, want)
        assert np.array_equal(H, J) == (len(set(dims)) == 1)


def test_dgn_until_first_dogleg():
    """Past a dogleg fallback the reference's path depends on last-bit rounding of
    the error (its first trial re-evaluates the rejected point, so the gain ratio
    is ±ε); the trajectory is therefore compared up to that event only."""
    g = load_golden("dgn_dogleg_L3")
    dims, R = [int(d) for d in g["dims"]], int(g["R"])
    o = _opts(g)
    np.random.seed(int(g["seed"]))
    _, ss, er, im, gr, st = orc.dGN(g["T"], split_x(g["init_x"], dims, R), R, o)
    ref = g["errors"]
    # iterations 6 and 7 trigger the fallback (error > 0.99 * previous error);
    # the outcome of the first is roundoff-independent, the second is not.
    np.testing.assert_allclose(er[:7], ref[:7], rtol=1e-8)


def test_dogleg_units():
    g = load_golden("dogleg_units")
    n = len(g["grad"])
    for row in g["rows"]:
        y, delta, want = row[:n], row[n], row[n + 1:]
        np.testing.assert_allclose(orc.dogleg(y, g["grad"], g["jtj"], delta), want, rtol=1e-12, atol=1e-14)
    T = g["T"]
    dims = list(T.shape)
    R = len(g["x"]) // sum(dims)
    bf, bx, by, be = orc.compute_dogleg_steps(np.linalg.norm(T), orc.unfold(T, 1),
                                              [np.zeros((d, R)) for d in dims], g["g2"], g["j2"],
                                              g["x"].copy(), g["y"].copy(), float(g["err"]), float(g["damp"]),
                                              False, 0)
    np.testing.assert_allclose(be, float(g["best_error"]), rtol=1e-10)
    np.testing.assert_allclose(bx, g["best_x"], rtol=1e-10, atol=1e-12)
    np.testing.assert_allclose(orc.cpd2flat(bf), g["best_f"], rtol=1e-10, atol=1e-12)


@pytest.mark.parametrize("name", ["mlsvd_seq", "mlsvd_classic", "mlsvd_seq_L4"])
def test_mlsvd_matches_reference(name):
    g = load_golden(name)
    T, R = g["T"], int(g["R"])
    o = orc.Options()
    o.mlsvd_method = str(g["method"])
    np.random.seed(int(g["seed"]))
    S, U, T1, sig = orc.mlsvd(T, np.linalg.norm(T), R, o)
    assert [u.shape[1] for u in U] == list(g["ranks"])
    np.testing.assert_allclose(np.concatenate(sig), g["sigmas"], rtol=1e-10)
    np.testing.assert_allclose(np.concatenate([u.flatten('F') for u in U]), g["U"], rtol=1e-8, atol=1e-10)
    np.testing.assert_allclose(S, g["S"], rtol=1e-8, atol=1e-9)


@pytest.mark.parametrize("name", ["cpd_c1_small", "cpd_L4", "cpd_refine", "cpd_symm", "cpd_symm_direct"])
def test_cpd_matches_reference(name):
    g = load_golden(name)
    o = _opts(g)
    np.random.seed(int(g["seed"]))
    f, out = orc.cpd(g["T"], int(g["R"]), o)
    assert out.num_steps == int(g["num_steps"])
    assert list(out.stop) == list(g["stop"])
    np.testing.assert_allclose(out.rel_error, float(g["rel_error"]), rtol=1e-6)
    np.testing.assert_allclose(np.concatenate([w.flatten('F') for w in f]), g["factors"], rtol=1e-6, atol=1e-8)


def test_sparse_units_match_reference():
    g = load_golden("sparse_L3")
    dims, R = [int(d) for d in g["dims"]], int(g["R"])
    W = split_x(g["W"], dims, R)
    fn = orc.sparse_fastnorm(g["data"], g["idxs"], dims, W)
    assert abs(fn - float(g["sparse_fastnorm"])) < 1e-12 * fn
    grams = []
    for l in range(3):
        Tl = orc.sparse_unfold(g["data"], g["idxs"], dims, l + 1)
        grams.append((Tl @ Tl.T).toarray().flatten())
    np.testing.assert_allclose(np.concatenate(grams), g["grams"], rtol=1e-13, atol=1e-13)
    UT, s = [], 0
    for l, n in enumerate(g["UT_rows"]):
        UT.append(g["UT"][s:s + n * dims[l]].reshape(n, dims[l]))
        s += n * dims[l]
    S = orc.sparse_multilin_mult(UT, g["data"], g["idxs"], dims)
    np.testing.assert_allclose(S, g["S"], rtol=1e-12, atol=1e-12)
    np.random.seed(41)
    f, out = orc.cpd([g["data"], g["idxs"], np.array(dims)], R)
    np.testing.assert_allclose(out.rel_error, float(g["cpd_rel_error"]), rtol=1e-6)


def test_reference_doctest_tensor():
    """tests/simple_tensor_cpd_options.py:8-35 of the reference, seeded."""
    g = load_golden("ref_tests_2x2x2")
    errs = []
    for seed in range(10):
        np.random.seed(seed)
        _, out = orc.cpd(g["T"], 3)
        errs.append(out.rel_error)
    np.testing.assert_allclose(errs, g["best_of_10"], rtol=1e-4, atol=1e-15)
    assert min(errs) < 1e-14
    o = orc.Options()
    o.initialization = [np.ones((2, 3))] * 3
    _, out = orc.cpd(g["T"], 3, o)
    np.testing.assert_allclose(out.rel_error, float(g["ones_init_error"]), rtol=1e-8)
    assert out.rel_error < 0.14


ALS_CASES = ["als_L3", "als_L4", "als_stall_L3", "als_symm_L3", "als_norm_L3"]


@pytest.mark.parametrize("name", ALS_CASES)
def test_als_trajectory_matches_reference(name):
    g = load_golden(name)
    dims, R = [int(d) for d in g["dims"]], int(g["R"])
    f, ss, er, im, gr, st = orc.als(g["T"], split_x(g["init_x"], dims, R), R, _opts(g))
    assert st == int(g["stop"])
    assert len(er) == len(g["errors"])
    np.testing.assert_allclose(er, g["errors"], rtol=1e-9, atol=1e-14)
    np.testing.assert_allclose(ss, g["step_sizes"], rtol=1e-9, atol=1e-14)
    np.testing.assert_allclose(im, g["improv"], rtol=1e-6, atol=1e-14)
    np.testing.assert_allclose(orc.cpd2flat(f), g["final_x"], rtol=1e-8, atol=1e-10)


@pytest.mark.parametrize("name", ["cpd_als", "cpd_als_refine"])
def test_cpd_als_matches_reference(name):
    g = load_golden(name)
    o = _opts(g)
    np.random.seed(int(g["seed"]))
    f, out = orc.cpd(g["T"], int(g["R"]), o)
    assert out.num_steps == int(g["num_steps"])
    assert list(out.stop) == list(g["stop"])
    np.testing.assert_allclose(out.rel_error, float(g["rel_error"]), rtol=1e-6)
    np.testing.assert_allclose(np.concatenate([w.flatten('F') for w in f]), g["factors"], rtol=1e-6, atol=1e-8)


def rank_tables(g):
    """The per-(rank, trial) error tables of a rank fixture."""
    t = int(g["trials"])
    out, s = [], 0
    for n in g["table_lens"]:
        out.append(g["tables"][s:s + n * t].reshape(n, t))
        s += n * t
    return out


@pytest.mark.parametrize("name", ["rank_rules_L3", "rank_rules_L4"])
def test_rank_rules_match_reference(name):
    g = load_golden(name)
    dims = [int(d) for d in g["dims"]]
    s = 0
    for k, tab in enumerate(rank_tables(g)):
        fr, epr = orc.rank(lambda r: float(np.min(tab[r - 1])), dims)
        n = int(g["error_lens"][k])
        assert fr == int(g["final_rank"][k])
        np.testing.assert_array_equal(epr, g["errors"][s:s + n])
        s += n


def test_smart_starts_match_reference():
    """Initialization.py:20-94 with 'smart_random' and 'smart' (Gaussian cores,
    integer cores with ties), including the RNG state left behind."""
    g = load_golden("init_smart")
    for k in range(int(g["n"])):
        S, R = g["S%d" % k], int(g["R%d" % k])
        for method in ("smart_random", "smart"):
            o = orc.Options()
            o.initialization = method
            o = orc.make_options(o)
            np.random.seed(int(g["seed"]) + k)
            f = orc.starting_point(S, [np.eye(d) for d in S.shape], R, list(range(S.ndim)), o)
            assert np.random.rand() == float(g["%s_after%d" % (method, k)])
            np.testing.assert_allclose(orc.cpd2flat(f), g["%s%d" % (method, k)], rtol=1e-12, atol=1e-15)


@pytest.mark.parametrize("name", ["cpd_smart", "cpd_smart_random"])
def test_cpd_smart_matches_reference(name):
    g = load_golden(name)
    o = _opts(g)
    np.random.seed(int(g["seed"]))
    f, out = orc.cpd(g["T"], int(g["R"]), o)
    assert out.num_steps == int(g["num_steps"])
    assert list(out.stop) == list(g["stop"])
    np.testing.assert_allclose(out.rel_error, float(g["rel_error"]), rtol=1e-6)


def test_tt_cores_match_reference():
    """cpdtt (TensorFox.py:1042-1065) cores and the RNG state after them."""
    g = load_golden("tt_cores")
    for k in range(int(g["n"])):
        T, R = g["T%d" % k], int(g["R%d" % k])
        np.random.seed(int(g["seed"]) + k)
        G = orc.cpdtt(T, R)
        assert np.random.rand() == float(g["after%d" % k])
        assert len(G) == int(g["ncores%d" % k])
        for j, c in enumerate(G):
            np.testing.assert_allclose(c, g["G%d_%d" % (k, j)], rtol=1e-9, atol=1e-11)


def congruence(A, B):
    """Smallest over matched columns of the product over modes of |cos|."""
    from scipy.optimize import linear_sum_assignment
    R = A[0].shape[1]
    C = np.ones((R, R))
    for a, b in zip(A, B):
        C *= np.abs((a / np.linalg.norm(a, axis=0)).T @ (b / np.linalg.norm(b, axis=0)))
    r, c = linear_sum_assignment(-C)
    return C[r, c].min()


@pytest.mark.parametrize("name", ["cpd_tt_L3", "cpd_tt_L4", "cpd_tt_L5", "cpd_tt_dgn_L4"])
def test_cpd_tt_matches_reference(name):
    """End to end, the tensor-train path is pinned by its result: the inner TT
    cores have orthonormal unfoldings, so the MLSVD basis of those modes is
    arbitrary and last-bit differences in a core rotate the compressed problem
    (the reference itself lands on the same solution with its columns permuted
    when a core changes by 1e-15).  The TT-SVD is pinned exactly above."""
    g = load_golden(name)
    o = _opts(g)
    o.method = 'ttcpd'
    np.random.seed(int(g["seed"]))
    f, out = orc.cpd(g["T"], int(g["R"]), o)
    assert abs(out.rel_error - float(g["rel_error"])) <= 1e-2 * float(g["rel_error"])
    T, R = g["T"], int(g["R"])
    assert congruence(f, split_x(g["factors"], T.shape, R)) > 0.999
    assert congruence(f, split_x(g["planted"], T.shape, R)) > 0.999
