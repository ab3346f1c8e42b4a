"""spdepy_gb300: GB300-native inference hot path of spdepy.

Q(theta) assembly, nested-dissection multifrontal Cholesky, log-determinants,
multi-RHS solves, selected inversion and the adjoint log-likelihood gradient run
in ``libspde_gb300`` (hand-written CUDA for sm_103a behind a C ABI); this package
mirrors the reference's Python API (``spdepy.grid``, ``spdepy.model``,
``Model``, ``spde_init``).
"""
from .grids import Grid, grid
from .model import Model
from .spdes import spde_init

__all__ = ["grid", "Grid", "model", "Model", "spde_init", "loglike"]


def loglike(model, par, grad_mode="exact"):
    """Differentiable log-likelihood objective (torch.autograd.Function)."""
    from .autograd import loglike as _ll
    return _ll(model, par, grad_mode)


def model(**kwargs) -> Model:
    """Model factory with the reference's keyword interface (reference ``__init__.py:13-53``):
    grid, spde, parameters, bc (default 3), ha (default True), anisotropic
    (default True), mod0; plus precision ("mixed" default, or "fp64")."""
    g = kwargs.get("grid")
    assert g is not None, "Grid is not defined"
    ha = kwargs.get("ha") if isinstance(kwargs.get("ha"), bool) else True
    bc = kwargs.get("bc") if isinstance(kwargs.get("bc"), int) else 3
    ani = kwargs.get("anisotropic") if isinstance(kwargs.get("anisotropic"), bool) else True
    precision = kwargs.get("precision", "mixed")
    mod0 = kwargs.get("mod0")
    if g.T > 1 and mod0 is None:
        mod0 = spde_init("whittle-matern", g.spatial(), ani=ani, ha=ha, bc=bc, precision=precision)
    elif mod0 is not None and hasattr(mod0, "mod"):
        mod0 = mod0.mod
    return Model(spde=kwargs.get("spde"), grid=g, parameters=kwargs.get("parameters"), ani=ani, ha=ha, bc=bc,
                 mod0=mod0, precision=precision)
