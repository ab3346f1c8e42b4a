"""Load the committed reference fixtures and rebuild matching oracle objects."""
import glob
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def model_cases():
    return sorted(os.path.basename(p)[6:-4] for p in glob.glob(os.path.join(GOLDEN, "model_*.npz")))


def separable_cases():
    """Separable space-time fixtures (the oracle and the CUDA path's 75-slot plans)."""
    return sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN, "separable_*.npz")))


def load(name):
    if not name.endswith(".npz"):
        name = name + ".npz" if name.startswith("separable_") else f"model_{name}.npz"
    return np.load(os.path.join(GOLDEN, name), allow_pickle=False)


def diff_form(g):
    return "ha" if int(g["ha"]) else ("ani" if int(g["ani"]) else "iso")


def grid_args(g):
    M, N, T, Nbs, ext = (int(g[k]) for k in ("M", "N", "T", "Nbs", "extend"))
    return dict(x=np.arange(M, dtype=float), y=np.arange(N, dtype=float),
                t=None if T == 1 else np.arange(T, dtype=float), extend=None if ext < 0 else ext, Nbs=Nbs)


def oracle_model(g):
    from oracle.spde_oracle import OracleGrid, OracleModel
    grid = OracleGrid(**grid_args(g))
    ww = g["ww"] if "ww" in g.files else None
    return OracleModel(grid, str(g["family"]), diff_form(g), int(g["bc"]), ww=ww)


def separable_oracle(g):
    from oracle.spde_oracle import OracleGrid, SeparableOracleModel
    return SeparableOracleModel(OracleGrid(**grid_args(g)), diff_form(g), int(g["bc"]), temporal=str(g["temporal"]))
