"""The optimiser loop (reference optim/__init__.py:26-62 and the step rules in
optim/*.py) against the reference's own trajectories on a fixed smooth
objective (tests/golden/optim.npz, made by tests/golden/make_golden.py)."""
import os
import sys

import numpy as np
import pytest

from golden_cases import load

sys.path.insert(0, os.path.join(os.path.dirname(__file__), "golden"))


def _objective(x):
    from make_golden import optim_objective
    return optim_objective(x)


def _runs():
    from make_golden import OPTIM_RUNS
    return OPTIM_RUNS


@pytest.mark.parametrize("i", range(9))
def test_step_rules_follow_the_reference(i):
    from spdepy_gb300.optim import Optimize
    g = load("optim.npz")
    step, kw = _runs()[i]
    assert str(g[f"r{i}_step"]) == step
    kw = dict(kw)
    kw["lr"] = np.asarray(kw["lr"], dtype=float)
    if "fix" in kw:
        kw["fix"] = np.asarray(kw["fix"])
    opt = Optimize(fun=_objective)
    res = opt.fit(x0=g["x0"].copy(), stepType=step, **kw)
    hist = np.array(opt.histX)
    assert hist.shape == g[f"r{i}_hist"].shape
    assert np.allclose(hist, g[f"r{i}_hist"], rtol=1e-12, atol=1e-14), np.abs(hist - g[f"r{i}_hist"]).max()
    assert np.allclose(opt.histF, g[f"r{i}_histf"], rtol=1e-12, atol=1e-14)
    assert np.allclose(res["x"], g[f"r{i}_x"], rtol=1e-12, atol=1e-14)
    assert res["fun"] == pytest.approx(float(g[f"r{i}_fun"]), rel=1e-12)
    assert res["method"] == step


def test_scalar_learning_rate_equals_a_constant_schedule():
    """A scalar lr (which the reference's loop cannot take) gives the run of the
    constant schedule."""
    from spdepy_gb300.optim import Optimize
    g = load("optim.npz")
    a = Optimize(fun=_objective).fit(x0=g["x0"].copy(), stepType="adam", lr=0.05, max_steps=40, pol=10)
    assert np.allclose(a["x"], g["r0_x"], rtol=1e-12, atol=1e-14)


def test_unknown_step_rule_is_refused():
    from spdepy_gb300.optim import Optimize
    with pytest.raises(ValueError, match="not recognized"):
        Optimize(fun=_objective).fit(x0=np.zeros(5), stepType="newton", lr=[0.1])


def test_verbose_prints_the_reference_progress_line(capsys):
    from spdepy_gb300.optim import Optimize
    g = load("optim.npz")
    Optimize(fun=_objective).fit(x0=g["x0"].copy(), stepType="adam", lr=[0.05] * 3, pol=2, verbose=True,
                                 print=lambda x: "x0 = %.2f" % x[0])
    out = capsys.readouterr().out.splitlines()
    assert len(out) == 3 and out[0].startswith("#   ") and "| fun = " in out[0] and "x0 = 1.00" in out[0]
