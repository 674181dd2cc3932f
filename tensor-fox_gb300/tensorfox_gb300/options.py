"""Options object with Tensor Fox's defaults (Auxiliar.py:242-362).

``make_options`` copies every attribute the caller's object defines over the
defaults, exactly like the reference.  Three fields are added by this package and
ignored by the reference: ``precision`` ('fp64', 'fp32' or None for the input's
own type, 'mixed' = FP32 data with TF32 tensor-core contractions for the
compression), ``cluster`` (CTAs per problem in the device engine, None = auto)
``tile`` (the engine's register tile, 1, 2 or 4; None = chosen by size, or by
the autotuner in ``cpd_batch``) and ``sparse_solver`` (None = the reference's
path for a COO tensor: compression, then dGN on the dense core; 'direct' = dGN
on the COO tensor itself, gradient and error from COO MTTKRPs).
"""

_DEFAULTS = dict(maxiter=200, tol=1e-16, tol_step=1e-6, tol_improv=1e-6, tol_grad=1e-6, tol_jump=10,
                 method='dGN', inner_method='cg', cg_maxiter=100, cg_factor=1, cg_tol=1e-16,
                 initialization='random', trunc_dims=0, mlsvd_method='seq', tol_mlsvd=1e-16, init_damp=1,
                 refine=False, symm=False, factors_norm=0, trials=3, display=0, epochs=1, gpu=False,
                 mkl_dot=True, svd_n_components=None, precision=None, cluster=None, tile=None,
                 sparse_solver=None)


class Options:
    """Attribute bag; ``make_options`` returns one with every field set."""

    def __repr__(self):
        return "Options(%s)" % ", ".join("%s=%r" % (k, getattr(self, k)) for k in _DEFAULTS)


def make_options(options=None):
    out = Options()
    for k, v in _DEFAULTS.items():
        setattr(out, k, v)
    out.bi_method_parameters = ['als', 500, 1e-6]
    if options is None or options is False:
        return out
    names = dir(options)
    for k in _DEFAULTS:
        if k in names:
            setattr(out, k, getattr(options, k))
    if 'bi_method' in names:
        out.bi_method_parameters[0] = options.bi_method
        out.bi_method_parameters[1] = {'cg': 1, 'cg_static': 100, 'als': 500}.get(options.bi_method, 500)
    if 'bi_method_maxiter' in names:
        out.bi_method_parameters[1] = options.bi_method_maxiter
    if 'bi_method_tol' in names:
        out.bi_method_parameters[2] = options.bi_method_tol
    if out.gpu and 'mlsvd_method' not in names:
        out.mlsvd_method = 'gpu'
    return out
