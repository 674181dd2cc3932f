"""Generates the golden fixtures in this folder by running the reference itself.

Run from the repository root, in a container where the reference source tree is
mounted, with TFX_REFERENCE_MODULES naming its ``modules`` directory (see
``ref_harness.py``):

    TFX_REFERENCE_MODULES=<reference>/modules python tests/golden/make_golden.py [case ...]

With case names, only those fixtures are regenerated (see ``CASES``).
Each ``.npz`` holds seeded inputs and the reference's outputs for one case.  The
fixtures are small (a few hundred KB in total) and committed; tests compare both
the oracle (``oracle/tfx_oracle.py``) and the CUDA path against them.
"""
import io
import contextlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
from ref_harness import load_reference  # noqa: E402

tfx = load_reference()
import TensorFox.GaussNewton as gn  # noqa: E402
import TensorFox.Conversion as cnv  # noqa: E402
import TensorFox.Critical as crt  # noqa: E402
import TensorFox.Compression as cmpr  # noqa: E402
import TensorFox.MultilinearAlgebra as mla  # noqa: E402
import TensorFox.Alternating_Least_Squares as alsm  # noqa: E402
import TensorFox.Initialization as ini  # noqa: E402


def save(name, **arrays):
    path = os.path.join(HERE, name + ".npz")
    np.savez_compressed(path, **{k: np.asarray(v) for k, v in arrays.items()})
    print("wrote", path)


def planted(dims, R, noise, seed):
    rng = np.random.default_rng(seed)
    W = [rng.standard_normal((d, R)) for d in dims]
    T = cnv.cpd2tens([w.copy() for w in W])
    if noise:
        E = rng.standard_normal(T.shape)
        T = T + noise * np.linalg.norm(T) / np.linalg.norm(E) * E
    return T, W


def units(name, dims, R, seed, damp=0.7, cg_iters=6):
    """gramians / regularization / precond / grad / matvec / cg on seeded inputs."""
    rng = np.random.default_rng(seed)
    L = len(dims)
    T = rng.standard_normal(dims)
    W = [rng.standard_normal((d, R)) for d in dims]
    v = rng.standard_normal(R * sum(dims))
    data = gn.prepare_data(dims, R)
    Gr, P1, P2, A, B, P_VT_W, result, result_tmp, Gamma, gamma, sum_dims, M, rc, P, Q, z, g, JtJg, N, gg = data
    Gr, P1, P2 = gn.gramians([w.copy() for w in W], Gr, P1, P2)
    Gamma, gamma = gn.regularization(Gamma, gamma, P1, np.array(dims), sum_dims)
    M = gn.precond(Gamma, gamma, M.copy(), damp, np.array(dims), sum_dims)
    Tl = [cnv.unfold_C(T, l + 1) for l in range(L)]
    grad = gn.compute_grad(Tl, [w.copy() for w in W], P1, g.copy(), N, gg, np.array(dims), sum_dims).copy()
    V = [v[sum_dims[l]:sum_dims[l + 1]].reshape(R, dims[l]) for l in range(L)]
    for l in range(L):
        np.dot(V[l], W[l], out=A[l])
        np.dot(V[l].T, P1[l], out=B[l])
    mv = gn.matvec([w.copy() for w in W], P2, P_VT_W, result, result_tmp, z.copy(), A, B, np.array(dims), sum_dims).copy()
    data = gn.prepare_data(dims, R)
    y0 = np.zeros(R * sum(dims))
    y, cgrad, jtj, itn, rn = gn.cg(Tl, [w.copy() for w in W], data, y0, damp, cg_iters, 0.0)
    T1a = np.empty(Tl[0].shape)
    T1a = cnv.cpd2unfold1(T1a, [w.copy() for w in W])
    fn = crt.fastnorm(Tl[0], T1a)
    x = np.concatenate([w.flatten('F') for w in W])
    eqf = cnv.x2cpd(x.copy() * 1.5, [w.copy() for w in W])
    save(name, dims=np.array(dims), R=R, T=T, x=x, v=v, damp=damp, cg_iters=cg_iters,
         Gr=Gr, P1=P1, P2=P2, Gamma=Gamma, gamma=gamma, M=M, grad=grad, matvec=mv,
         cg_y=y, cg_grad=cgrad, cg_jtj=jtj, cg_itn=itn, cg_rn=rn, T1_approx=T1a, fastnorm=fn,
         eq_x=np.concatenate([f.flatten('F') for f in eqf]))


class Opt:
    pass


def dgn_case(name, dims, R, seed, noise=1e-3, fix=-1, alias=False, symmetric=False, **opts):
    """dGN trajectory from an explicit start; 'cg' budgets replayed from a fixed seed.
    ``fix`` >= 0 passes that factor as ``[W]`` (kept fixed, as bicpd does);
    ``alias`` passes ONE array for every mode (as a symmetric start is);
    ``symmetric`` plants a symmetric tensor."""
    T, W = planted(dims, R, noise, seed)
    if symmetric:
        T = cnv.cpd2tens([W[0]] * len(dims)) + noise * np.random.default_rng(seed + 7).standard_normal(dims)
        W = [W[0]] * len(dims)
    rng = np.random.default_rng(seed + 1000)
    init = [w + 0.3 * rng.standard_normal(w.shape) for w in W]
    if alias:
        init = [init[0]] * len(dims)
    o = Opt()
    for k, v in opts.items():
        setattr(o, k, v)
    o = tfx.make_options(o)
    np.random.seed(seed)
    start = [init[0].copy()] * len(dims) if alias else [w.copy() for w in init]
    if fix >= 0:
        start[fix] = [start[fix]]
    bf, ss, er, im, gr, st = gn.dGN(T, start, R, o)
    save(name, T=T, init_x=np.concatenate([w.flatten('F') for w in init]), R=R, seed=seed, fix=fix, alias=int(alias),
         dims=np.array(dims), best_x=np.concatenate([w.flatten('F') for w in bf]),
         step_sizes=ss, errors=er, improv=im, gradients=gr, stop=st,
         opt_names=np.array(list(opts.keys())), opt_values=np.array([repr(v) for v in opts.values()]))


def mlsvd_case(name, dims, R, seed, method='seq', noise=1e-2):
    T, _ = planted(dims, R, noise, seed)
    o = Opt()
    o.mlsvd_method = method
    o = tfx.make_options(o)
    np.random.seed(seed)
    S, U, T1, sig = cmpr.mlsvd(T, np.linalg.norm(T), R, o)
    save(name, T=T, R=R, seed=seed, S=S, sigmas=np.concatenate(sig),
         ranks=np.array([u.shape[1] for u in U]), U=np.concatenate([u.flatten('F') for u in U]),
         method=method)


def cpd_case(name, dims, R, seed, noise, symmetric=False, **opts):
    T, W = planted(dims, R, noise, seed)
    if symmetric:
        T = cnv.cpd2tens([W[0]] * len(dims)) + noise * np.random.default_rng(seed + 7).standard_normal(dims)
        W = [W[0]] * len(dims)
    o = Opt()
    for k, v in opts.items():
        setattr(o, k, v)
    np.random.seed(seed)
    f, out = tfx.cpd(T, R, o)
    save(name, T=T, R=R, seed=seed, planted=np.concatenate([w.flatten('F') for w in W]),
         factors=np.concatenate([w.flatten('F') for w in f]), rel_error=out.rel_error,
         num_steps=out.num_steps, errors=out.errors[0], stop=np.array(out.stop),
         opt_names=np.array(list(opts.keys())), opt_values=np.array([repr(v) for v in opts.values()]))


def sparse_case(name, dims, R, nnz, seed):
    rng = np.random.default_rng(seed)
    L = len(dims)
    lin = rng.choice(int(np.prod(dims)), size=nnz, replace=False)
    idxs = np.stack(np.unravel_index(lin, dims), axis=1).astype(np.int64)
    W = [rng.standard_normal((d, R)) for d in dims]
    vals = np.ones(nnz)
    for l in range(L):
        vals = vals * 0 + vals  # keep dtype
    model = np.ones((nnz, R))
    for l in range(L):
        model *= W[l][idxs[:, l]]
    data = model.sum(1) + 0.01 * rng.standard_normal(nnz)
    fnorm = crt.sparse_fastnorm(data, idxs.astype(np.uint64), np.array(dims), [w.copy() for w in W])
    grams = []
    for l in range(L):
        Tl = cnv.sparse_unfold(data, idxs.astype(np.uint64), np.array(dims), l + 1)
        grams.append((Tl @ Tl.T).toarray().flatten())
    UT = [rng.standard_normal((min(R + 1, d), d)) for d in dims]
    S = mla.sparse_multilin_mult([u.copy() for u in UT], data, idxs.astype(np.uint64), np.array(dims))
    np.random.seed(seed)
    f, out = tfx.cpd([data, idxs, np.array(dims)], R)
    save(name, dims=np.array(dims), R=R, idxs=idxs, data=data, W=np.concatenate([w.flatten('F') for w in W]),
         sparse_fastnorm=fnorm, grams=np.concatenate(grams), UT=np.concatenate([u.flatten() for u in UT]),
         UT_rows=np.array([u.shape[0] for u in UT]), S=S, cpd_rel_error=out.rel_error,
         cpd_factors=np.concatenate([w.flatten('F') for w in f]), cpd_stop=np.array(out.stop))


def dogleg_units(name, seed):
    """dogleg() on every branch and compute_dogleg_steps() from a long step (‖y‖ > delta)."""
    rng = np.random.default_rng(seed)
    n = 30
    rows = []
    grad = rng.standard_normal(n)
    H = rng.standard_normal((n, n))
    H = H @ H.T + n * np.eye(n)
    jtj = H @ grad
    for scale, delta in [(0.01, 1.0), (5.0, 0.001), (5.0, 1.0), (5.0, 3.0), (2.0, 0.2)]:
        y = scale * rng.standard_normal(n)
        rows.append(np.concatenate([y, [delta], gn.dogleg(y, grad, jtj, delta)]))
    dims, R = [7, 6, 5], 3
    T, W = planted(dims, R, 0.05, seed)
    Tl = [cnv.unfold_C(T, l + 1) for l in range(3)]
    x = np.concatenate([w.flatten('F') for w in W]) + 0.05 * rng.standard_normal(R * sum(dims))
    y = 4.0 * rng.standard_normal(R * sum(dims))
    g2 = rng.standard_normal(R * sum(dims))
    j2 = 50 * g2 + rng.standard_normal(R * sum(dims))
    factors = [np.zeros((d, R)) for d in dims]
    err = 10.0
    ip = (0.3, 'cg', 100, 1, 1e-16, 10, False, 0, -1)
    bf, bx, by, be = gn.compute_dogleg_steps(np.linalg.norm(T), Tl, np.empty(Tl[0].shape), factors, g2, j2,
                                             x.copy(), y.copy(), err, ip)
    save(name, grad=grad, jtj=jtj, rows=np.array(rows), T=T, x=x, y=y, g2=g2, j2=j2, err=err, damp=0.3,
         best_x=bx, best_y=by, best_error=be, best_f=np.concatenate([f.flatten('F') for f in bf]))


def kr_case(name, seed):
    rng = np.random.default_rng(seed)
    A, B = rng.standard_normal((4, 3)), rng.standard_normal((5, 3))
    M = mla.khatri_rao(A, B, np.empty((20, 3)))
    T = rng.standard_normal((4, 3, 5, 2))
    unf = [cnv.unfold(T, m + 1) for m in range(4)]
    save(name, A=A, B=B, KR=M, T=T, unf=np.concatenate([u.flatten() for u in unf]))


def reference_tests_case(name):
    """The 2x2x2 tensor of tests/simple_tensor_cpd_options.py:8-15 at R=3 and options."""
    m = 2
    T = np.zeros((m, m, m))
    s = 0
    for k in range(m):
        for i in range(m):
            for j in range(m):
                T[i, j, k] = s
                s += 1
    errs = []
    for seed in range(10):
        np.random.seed(seed)
        f, out = tfx.cpd(T, 3)
        errs.append(out.rel_error)
    o = Opt()
    o = tfx.make_options(o)
    o.initialization = [np.ones((m, 3))] * 3
    np.random.seed(0)
    _, out_ones = tfx.cpd(T, 3, o)
    save(name, T=T, best_of_10=np.array(errs), ones_init_error=out_ones.rel_error,
         ones_init_errors=out_ones.errors[0])


def als_case(name, dims, R, seed, noise=1e-3, spread=0.3, **opts):
    """ALS trajectory (Alternating_Least_Squares.py:18-201) from an explicit start."""
    T, W = planted(dims, R, noise, seed)
    rng = np.random.default_rng(seed + 1000)
    init = [w + spread * rng.standard_normal(w.shape) for w in W]
    o = Opt()
    for k, v in opts.items():
        setattr(o, k, v)
    o = tfx.make_options(o)
    f, ss, er, im, gr, st = alsm.als(T, [w.copy() for w in init], R, o)
    save(name, T=T, init_x=np.concatenate([w.flatten('F') for w in init]), R=R, seed=seed,
         dims=np.array(dims), final_x=np.concatenate([w.flatten('F') for w in f]),
         step_sizes=ss, errors=er, improv=im, gradients=gr, stop=st,
         opt_names=np.array(list(opts.keys())), opt_values=np.array([repr(v) for v in opts.values()]))


def rank_case(name, dims, tables, trials=3):
    """TensorFox.py:820-939 rank(): the stopping rules, with cpd replaced by a table
    of relative errors per (rank, trial) so that only the driver logic runs."""
    L = len(dims)
    out_ranks, out_err, lens, flat = [], [], [], []
    for table in tables:
        calls = []

        def fake_cpd(T, r, options=False, _t=table, _c=calls):
            _c.append(r)
            k = sum(1 for x in _c if x == r) - 1

            class Out:
                pass
            o = Out()
            o.rel_error = float(_t[r - 1][k])
            return None, o
        mod = sys.modules["TensorFox.TensorFox"]
        real = mod.cpd
        mod.cpd = fake_cpd
        try:
            with contextlib.redirect_stdout(io.StringIO()):
                fr, epr = mod.rank(np.zeros(dims), plot=False, trials=trials)
        finally:
            mod.cpd = real
        out_ranks.append(fr)
        out_err.append(np.asarray(epr))
        lens.append(len(table))
        flat.append(np.asarray(table, dtype=np.float64).ravel())
    save(name, dims=np.array(dims), trials=trials, table_lens=np.array(lens), tables=np.concatenate(flat),
         final_rank=np.array(out_ranks), error_lens=np.array([len(e) for e in out_err]),
         errors=np.concatenate(out_err))


def rank_tables(L, n, trials, seed):
    """Seeded per-(rank, trial) error tables that exercise every stopping rule."""
    rng = np.random.default_rng(seed)
    tabs = []
    # error flattens (|e_r - e_{r-1}| < 1e-5, e < 0.5) after the true rank 4
    e = [0.9, 0.6, 0.3, 0.01, 0.01 - 4e-6, 0.01 - 5e-6]
    tabs.append([[x * (1 + 0.5 * t) for t in range(trials)] for x in e] + [[1.0] * trials] * (n - len(e)))
    # exact fit at rank 3 (error < 1e-14)
    e = [0.5, 0.2, 1e-15]
    tabs.append([[x, x * 2, x * 3] [:trials] for x in e] + [[1.0] * trials] * (n - len(e)))
    # abrupt drop: previous difference / current difference > 100
    e = [0.8, 0.4, 0.39, 1e-3, 1e-3 - 1e-6, 1e-3 - 2e-6]
    tabs.append([[x] * trials for x in e] + [[1.0] * trials] * (n - len(e)))
    # no rule fires: runs to Rmax, final rank = argmin
    e = list(np.sort(rng.uniform(0.6, 0.9, n))[::-1] + np.arange(n) * 1e-3)
    tabs.append([[x + 1e-3 * t for t in range(trials)] for x in e])
    # the flat-error rule with error >= 0.5 does not fire
    e = [0.9, 0.7, 0.7 - 1e-6, 0.3, 0.05, 0.05 - 1e-6]
    tabs.append([[x] * trials for x in e] + [[1.0] * trials] * (n - len(e)))
    return tabs


def init_case(name, seed):
    """starting_point (Initialization.py:20-94) with 'smart_random' and 'smart' on
    seeded cores (Gaussian, and integer-valued with ties), with the RNG state it
    leaves (np.random.rand() drawn right after)."""
    rng = np.random.default_rng(seed)
    rows = []
    cores = [((5, 4, 3), 3, rng.standard_normal((5, 4, 3))),
             ((6, 5, 4), 4, rng.standard_normal((6, 5, 4))),
             ((4, 4, 3, 3), 2, rng.standard_normal((4, 4, 3, 3))),
             ((5, 4, 3), 4, rng.integers(-3, 4, size=(5, 4, 3)).astype(np.float64)),
             ((4, 3, 3), 6, np.arange(36, dtype=np.float64).reshape(4, 3, 3) % 5 - 2.0)]
    out = {}
    for k, (dims, R, S) in enumerate(cores):
        for method in ("smart_random", "smart"):
            o = Opt()
            o.initialization = method
            o = tfx.make_options(o)
            np.random.seed(seed + k)
            f = ini.starting_point(S, 1.0, S, [np.eye(d) for d in dims], R, list(range(len(dims))), o)
            after = np.random.rand()
            out["S%d" % k] = S
            out["R%d" % k] = R
            out["%s%d" % (method, k)] = np.concatenate([w.flatten('F') for w in f])
            out["%s_after%d" % (method, k)] = after
    out["n"] = len(cores)
    out["seed"] = seed
    save(name, **out)


def tt_case(name, shapes, seed):
    """cpdtt (TensorFox.py:1042-1065, tt_core Auxiliar.py:365-380): the TT cores
    of seeded tensors and the RNG state the randomized SVDs leave behind."""
    tf_mod = sys.modules["TensorFox.TensorFox"]
    rng = np.random.default_rng(seed)
    out = {"n": len(shapes), "seed": seed}
    for k, (dims, R) in enumerate(shapes):
        T = rng.standard_normal(dims)
        np.random.seed(seed + k)
        G = tf_mod.cpdtt(T, R)
        out["T%d" % k] = T
        out["R%d" % k] = R
        out["ncores%d" % k] = len(G)
        for j, g in enumerate(G):
            out["G%d_%d" % (k, j)] = g
        out["after%d" % k] = np.random.rand()
    save(name, **out)


def cpd_tt_case(name, dims, R, seed, noise, **opts):
    """cpd with method='ttcpd' (TensorFox.py:256-421 highcpd, 658-817 bicpd,
    Auxiliar.py:413-527 cpd_cores)."""
    T, W = planted(dims, R, noise, seed)
    o = Opt()
    o.method = 'ttcpd'
    for k, v in opts.items():
        setattr(o, k, v)
    np.random.seed(seed)
    f, out = tfx.cpd(T, R, o)
    save(name, T=T, R=R, seed=seed, planted=np.concatenate([w.flatten('F') for w in W]),
         factors=np.concatenate([w.flatten('F') for w in f]), rel_error=out.rel_error,
         num_steps=out.num_steps, core_steps=np.array([c.num_steps for c in out.cpd_output]),
         core_errors=np.array([c.rel_error for c in out.cpd_output]), after=np.random.rand(),
         opt_names=np.array(list(opts.keys())), opt_values=np.array([repr(v) for v in opts.values()]))


def cpd_tt_sparse_case(name, dims, R, nnz, seed):
    """cpd with method='ttcpd' on a COO tensor sampled from a planted model."""
    rng = np.random.default_rng(seed)
    L = len(dims)
    lin = rng.choice(int(np.prod(dims)), size=nnz, replace=False)
    idxs = np.stack(np.unravel_index(lin, dims), axis=1).astype(np.int64)
    W = [rng.standard_normal((d, R)) for d in dims]
    model = np.ones((nnz, R))
    for l in range(L):
        model *= W[l][idxs[:, l]]
    data = model.sum(1) + 1e-3 * rng.standard_normal(nnz)
    o = Opt()
    o.method = 'ttcpd'
    np.random.seed(seed)
    f, out = tfx.cpd([data, idxs, np.array(dims)], R, o)
    save(name, dims=np.array(dims), R=R, seed=seed, idxs=idxs, data=data,
         factors=np.concatenate([w.flatten('F') for w in f]), rel_error=out.rel_error, num_steps=out.num_steps)


def consistency_case(name):
    """Auxiliar.py:24-78: the reference's SystemExit message for each invalid
    input (an empty string where the input is accepted)."""
    aux = sys.modules["TensorFox.Auxiliar"]
    cases = [((3, 3, 3), 2, {}), ((2,) * 13, 2, {}), ((4, 1, 3), 2, {}), ((4, 3, 3), 0, {}), ((4, 3, 3), 2.0, {}),
             ((4, 3, 3), 10, {}), ((4, 3, 3), 9, {}), ((4, 3, 3, 2), 1, {}), ((4, 4, 4), 2, {"symm": True}),
             ((4, 3, 4), 2, {"symm": True}), ((4, 3, 3), 2, {"method": "foo"}), ((2,) * 12, 2, {})]
    msgs = []
    for dims, R, opts in cases:
        o = Opt()
        for k, v in opts.items():
            setattr(o, k, v)
        o = tfx.make_options(o)
        try:
            aux.consistency(R, dims, o)
            msgs.append("")
        except SystemExit as e:
            msgs.append(str(e))
    save(name, dims=np.array([repr(c[0]) for c in cases]), ranks=np.array([repr(c[1]) for c in cases]),
         opts=np.array([repr(c[2]) for c in cases]), msgs=np.array(msgs))


CASES = {
    "consistency": lambda: consistency_case("consistency"),
    "cpd_overrank": lambda: cpd_case("cpd_overrank", [6, 5, 4], 7, 76, 1e-4),
    "cpd_tt_sparse": lambda: cpd_tt_sparse_case("cpd_tt_sparse", [8, 7, 6, 5], 2, 1680, 75),
    "tt_cores": lambda: tt_case("tt_cores", [((6, 5, 4, 3), 2), ((5, 4, 4, 3, 3), 2), ((7, 6, 5, 4), 3)], 71),
    "cpd_tt_L4": lambda: cpd_tt_case("cpd_tt_L4", [9, 8, 7, 6], 3, 72, 1e-5),
    "cpd_tt_L5": lambda: cpd_tt_case("cpd_tt_L5", [7, 6, 6, 5, 5], 2, 73, 1e-5),
    "cpd_tt_dgn_L4": lambda: cpd_tt_case("cpd_tt_dgn_L4", [9, 8, 7, 6], 3, 76, 1e-5, bi_method='cg_static',
                                         inner_method='cg_static', cg_maxiter=10, maxiter=60),
    "dgn_fix_cg_L3": lambda: dgn_case("dgn_fix_cg_L3", [8, 7, 6], 3, 37, fix=2, inner_method='cg_static',
                                      cg_maxiter=8, maxiter=30),
    "dgn_fix_cgr_L3": lambda: dgn_case("dgn_fix_cgr_L3", [9, 8, 7], 3, 38, fix=1, maxiter=40),
    "cpd_tt_L3": lambda: cpd_tt_case("cpd_tt_L3", [10, 9, 8], 3, 74, 1e-5),
    "init_smart": lambda: init_case("init_smart", 61),
    "cpd_smart": lambda: cpd_case("cpd_smart", [14, 12, 10], 3, 62, 1e-5, initialization='smart'),
    "cpd_smart_random": lambda: cpd_case("cpd_smart_random", [14, 12, 10], 3, 63, 1e-5,
                                         initialization='smart_random'),
    "units_L3": lambda: units("units_L3", [7, 5, 4], 3, 1),
    "units_L4": lambda: units("units_L4", [5, 4, 3, 3], 2, 2),
    "units_L3_big": lambda: units("units_L3_big", [12, 10, 9], 4, 3, damp=0.2, cg_iters=9),
    "units_L5": lambda: units("units_L5", [4, 3, 3, 2, 2], 3, 4),
    "kr_unfold": lambda: kr_case("kr_unfold", 5),
    "dogleg_units": lambda: dogleg_units("dogleg_units", 6),
    "dgn_static_L3": lambda: dgn_case("dgn_static_L3", [9, 8, 7], 3, 11, inner_method='cg_static', cg_maxiter=8,
                                      maxiter=40),
    "dgn_cg_L3": lambda: dgn_case("dgn_cg_L3", [12, 10, 9], 4, 12, maxiter=60),
    "dgn_cg_L4": lambda: dgn_case("dgn_cg_L4", [6, 5, 5, 4], 3, 13, maxiter=50),
    "dgn_dogleg_L3": lambda: dgn_case("dgn_dogleg_L3", [8, 7, 6], 3, 14, noise=0.2, tol_jump=0.99, maxiter=30),
    "dgn_small_L3": lambda: dgn_case("dgn_small_L3", [4, 4, 3], 2, 15, maxiter=80),
    "dgn_als_L3": lambda: dgn_case("dgn_als_L3", [9, 8, 7], 3, 16, inner_method='als', maxiter=40),
    "dgn_als_L4": lambda: dgn_case("dgn_als_L4", [6, 5, 5, 4], 3, 17, inner_method='als', maxiter=40),
    "dgn_als_fix_L3": lambda: dgn_case("dgn_als_fix_L3", [8, 7, 6], 3, 18, fix=0, inner_method='als', maxiter=30),
    "dgn_direct_L3": lambda: dgn_case("dgn_direct_L3", [9, 8, 7], 3, 19, inner_method='direct', maxiter=30),
    "dgn_direct_L4": lambda: dgn_case("dgn_direct_L4", [6, 5, 5, 4], 3, 20, inner_method='direct', maxiter=30),
    "dgn_direct_fix_L3": lambda: dgn_case("dgn_direct_fix_L3", [8, 7, 6], 3, 24, fix=1, inner_method='direct',
                                          maxiter=25),
    "dgn_direct_symm_L3": lambda: dgn_case("dgn_direct_symm_L3", [6, 6, 6], 2, 25, inner_method='direct',
                                           maxiter=20, symm=True),
    "dgn_direct_big_L3": lambda: dgn_case("dgn_direct_big_L3", [20, 18, 16], 6, 26, noise=1e-2,
                                          inner_method='direct', maxiter=15),
    "dgn_symm_L3": lambda: dgn_case("dgn_symm_L3", [7, 7, 7], 3, 28, symmetric=True, inner_method='cg_static',
                                    cg_maxiter=6, maxiter=25, symm=True),
    "dgn_symm_alias_L3": lambda: dgn_case("dgn_symm_alias_L3", [7, 7, 7], 3, 29, symmetric=True, alias=True,
                                          inner_method='cg_static', cg_maxiter=6, maxiter=25, symm=True),
    "dgn_symm_norm_L3": lambda: dgn_case("dgn_symm_norm_L3", [6, 6, 6], 2, 30, symmetric=True, alias=True,
                                         inner_method='cg_static', cg_maxiter=6, maxiter=20, symm=True,
                                         factors_norm=3.0),
    "dgn_symm_direct_alias_L3": lambda: dgn_case("dgn_symm_direct_alias_L3", [6, 6, 6], 2, 34, symmetric=True,
                                                 alias=True, inner_method='direct', maxiter=15, symm=True),
    "cpd_symm": lambda: cpd_case("cpd_symm", [10, 10, 10], 3, 35, 1e-4, symmetric=True, symm=True, maxiter=60),
    "cpd_symm_direct": lambda: cpd_case("cpd_symm_direct", [8, 8, 8], 2, 36, 1e-4, symmetric=True, symm=True,
                                        inner_method='direct', maxiter=30),
    "dgn_damp_sched_L3": lambda: dgn_case("dgn_damp_sched_L3", [9, 8, 7], 3, 39, inner_method='cg_static',
                                          cg_maxiter=8, maxiter=25,
                                          init_damp=[float(0.5 * 0.8 ** k) for k in range(26)]),
    "dgn_norm_L3": lambda: dgn_case("dgn_norm_L3", [9, 8, 7], 3, 40, inner_method='cg_static', cg_maxiter=8,
                                    maxiter=25, factors_norm=2.0),
    "dgn_mixed_L3": lambda: dgn_case("dgn_mixed_L3", [9, 8, 7], 3, 27, inner_method=['direct'] * 4 + ['als'] * 26,
                                     maxiter=30),
    "mlsvd_seq": lambda: mlsvd_case("mlsvd_seq", [20, 15, 12], 4, 21),
    "mlsvd_classic": lambda: mlsvd_case("mlsvd_classic", [18, 14, 11], 3, 22, method='classic'),
    "mlsvd_seq_L4": lambda: mlsvd_case("mlsvd_seq_L4", [10, 9, 8, 7], 3, 23),
    "cpd_c1_small": lambda: cpd_case("cpd_c1_small", [30, 25, 20], 5, 31, 1e-6),
    "cpd_L4": lambda: cpd_case("cpd_L4", [12, 11, 10, 9], 3, 32, 1e-4),
    "cpd_refine": lambda: cpd_case("cpd_refine", [15, 12, 10], 4, 33, 1e-3, refine=True),
    "sparse_L3": lambda: sparse_case("sparse_L3", [10, 9, 8], 3, 60, 41),
    "ref_tests_2x2x2": lambda: reference_tests_case("ref_tests_2x2x2"),
    "als_L3": lambda: als_case("als_L3", [12, 10, 9], 4, 51, maxiter=60),
    "als_L4": lambda: als_case("als_L4", [7, 6, 5, 4], 3, 52, maxiter=80),
    "als_stall_L3": lambda: als_case("als_stall_L3", [9, 8, 7], 5, 53, noise=0.3, spread=1.0, maxiter=120),
    "als_symm_L3": lambda: als_case("als_symm_L3", [6, 6, 6], 3, 54, noise=1e-2, maxiter=30, symm=True),
    "als_norm_L3": lambda: als_case("als_norm_L3", [8, 7, 6], 3, 55, maxiter=30, factors_norm=2.0),
    "cpd_als": lambda: cpd_case("cpd_als", [20, 16, 12], 4, 56, 1e-5, method='als'),
    "cpd_als_refine": lambda: cpd_case("cpd_als_refine", [14, 12, 10], 3, 57, 1e-4, method='als', refine=True,
                                       maxiter=100),
    "rank_rules_L3": lambda: rank_case("rank_rules_L3", [4, 3, 3], rank_tables(3, 9, 3, 58)),
    "rank_rules_L4": lambda: rank_case("rank_rules_L4", [3, 3, 2, 2], rank_tables(4, 18, 2, 59), trials=2),
}


def main(names=None):
    for name in (names or list(CASES)):
        CASES[name]()


if __name__ == "__main__":
    main(sys.argv[1:])
