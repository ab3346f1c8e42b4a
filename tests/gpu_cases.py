"""Build GPU model objects matching the golden fixtures."""
import numpy as np

from golden_cases import diff_form, grid_args


def separable_gpu_model(g, precision="fp64"):
    """GPU model for a separable_* fixture (75-slot plan)."""
    from spdepy_gb300.grids import Grid
    from spdepy_gb300.spdes import spde_init
    ga = grid_args(g)
    grid = Grid(ga["x"], ga["y"], ga["t"], ga["extend"], ga["Nbs"])
    d = diff_form(g)
    mod = spde_init("seperable-spatial-temporal", grid, ani=d != "iso", ha=d == "ha", bc=int(g["bc"]),
                    precision=precision)
    mod.setPars(g["par"])
    mod.initFit(g["y"], idx=g["idx"])
    return mod


def gpu_model(g, precision="fp64"):
    from spdepy_gb300.grids import Grid
    from spdepy_gb300.spdes import _CLASSES
    ga = grid_args(g)
    grid = Grid(ga["x"], ga["y"], ga["t"], ga["extend"], ga["Nbs"])
    fam = str(g["family"])
    d = diff_form(g)
    bc = int(g["bc"])
    mod0 = None
    if grid.T > 1:
        mod0 = _CLASSES[("whittle-matern", d)](grid=grid.spatial(), bc=bc, precision=precision)
    ww = g["ww"] if "ww" in g.files else None
    mod = _CLASSES[(fam, d)](grid=grid, par=None, bc=bc, mod0=mod0, ww=ww, precision=precision)
    mod.setPars(g["par"])
    mod.initFit(g["y"], idx=g["idx"])
    return mod
