"""Every built option branch of the path against the oracle, both forms.

* filtering: Hou & Li and the 2/3 rule (inversion_utils.f90:377-455);
* viscosity prefactor (pretype): constant, vorch, max-strain,
  us-max-strain and roll-mean-max-strain, the reference default
  (advance.f90:381-410), with a 4-entry rolling window so the ring of
  rolling_mean.f90:36-69 wraps within the run;
* length scale of the viscosity: Kolmogorov and geophysical
  (inversion_utils.f90:124-218).

For each combination: the filter and hyperdiffusion tables and the initial
energy after setup_fields, adapt's time step and diagnostics at t = 0, and 20
impl-diff-rk4 steps with dt, the rolling mean and the prefactor compared per
step and the state at the end.  Tolerances: FP64 1e-12 (state), 1e-11
(diagnostics), 1e-10 (initial energy); mixed form 1e-6 (solenoidal state),
2e-5 (diagnostics), 2e-6 (initial energy, from the FP32 fields).  The
captured (CUDA-graph) step of the mixed form runs the prefactor logic on the
device; it is checked bitwise against the host-driven step for every pretype.
"""
import numpy as np
import pytest

import oracle
from ps3d_gb300 import Ps3dGpu
from tests.parity_util import beltrami_case, rel_l2

pytestmark = pytest.mark.gpu

PRETYPES = ["constant", "vorch", "max-strain", "us-max-strain", "roll-mean-max-strain"]
FILTERS = ["Hou & Li", "2/3-rule"]
LENGTHS = ["Kolmogorov", "geophysical"]
TOL = {"fp64": dict(state=1e-12, diag=1e-11, table=1e-13, energy=1e-10),
       "mixed": dict(state=1e-6, diag=2e-5, table=1e-13, energy=2e-6)}


def _pair(n, precision, **kw):
    lo, ex, vor, pert = beltrami_case(n, seed=7, amplitude=1e-2)
    cfg = dict(cflmax=0.5, roll_mean_win_size=4, **kw)
    o = oracle.Oracle(n, n, n, lo, ex, **cfg)
    g = Ps3dGpu(n, n, n, lo, ex, precision=precision, **cfg)
    te_o, en_o = o.setup_fields(vor, pert)
    te_g, en_g = g.setup_fields(vor, pert)
    return o, g, (te_o, en_o), (te_g, en_g)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("length_scale", LENGTHS)
@pytest.mark.parametrize("filtering", FILTERS, ids=["houli", "twothirds"])
@pytest.mark.parametrize("pretype", PRETYPES)
def test_option_branches_match_oracle(pretype, filtering, length_scale, precision):
    tol = TOL[precision]
    o, g, eo, eg = _pair(32, precision, pretype=pretype, filtering=filtering, length_scale=length_scale)
    # initial energy and enstrophy (FP32 velocity and vorticity in the mixed form)
    for a, b in zip(eg, eo):
        assert abs(a - b) <= tol["energy"] * abs(b), (a, b)
    assert rel_l2(g.table("filt"), o.table("filt")) < tol["table"]
    # the Kolmogorov viscosity scales with (te/en)^(1/3) of the set-up fields
    assert rel_l2(g.table("vhdis"), o.table("vhdis")) < tol["energy"]
    dtg, dg = g.adapt(0.0)
    dto, do = o.adapt(0.0)
    assert abs(dtg - dto) <= tol["diag"] * dto
    for k in ("ke", "en", "vorch", "ggmax", "usggmax", "lsggmax", "rmv", "pref"):
        assert abs(dg[k] - do[k]) <= tol["diag"] * max(abs(do[k]), 1e-300), (k, dg[k], do[k])
    # fresh pair for the run (adapt above advanced the rolling means)
    o, g, _, _ = _pair(32, precision, pretype=pretype, filtering=filtering, length_scale=length_scale)
    t_o = t_g = 0.0
    for s in range(20):
        t_g, dg = g.advance(t_g)
        t_o, do = o.advance(t_o)
        for k in ("dt", "rmv", "pref", "ke"):
            assert abs(dg[k] - do[k]) <= tol["diag"] * max(abs(do[k]), 1e-300), (s, k, dg[k], do[k])
    if precision == "mixed":
        # the mixed form keeps svor projected; the reference projects it at
        # the start of the next vor2vel
        o.vor2vel()
        g.vor2vel()
    err = rel_l2(g.get("svor"), o.get("svor"))
    assert err < tol["state"], err
    assert abs(t_g - t_o) <= tol["diag"] * t_o


@pytest.mark.parametrize("pretype", PRETYPES)
def test_captured_step_prefactor_logic_matches_host(pretype):
    """The device-side adapt scalars of the captured step (prefactor
    selection, rolling mean over a wrapping 4-entry window) against the
    host-driven advance, bitwise, over 8 steps."""
    a = Ps3dGpu(32, 32, 32, *beltrami_case(32, seed=8)[:2], precision="mixed", cflmax=0.5, pretype=pretype,
                roll_mean_win_size=4)
    b = Ps3dGpu(32, 32, 32, *beltrami_case(32, seed=8)[:2], precision="mixed", cflmax=0.5, pretype=pretype,
                roll_mean_win_size=4)
    _, _, vor, pert = beltrami_case(32, seed=8, amplitude=1e-2)
    a.setup_fields(vor, pert)
    b.setup_fields(vor, pert)
    t_a = 0.0
    for _ in range(8):
        t_a, d_a = a.advance(t_a)
    t_b, d_b, _ = b.advance_graph(0.0, 8)
    assert t_a == t_b
    for k in ("dt", "rmv", "pref", "ggmax", "usggmax", "vorch"):
        assert d_a[k] == d_b[k], (k, d_a[k], d_b[k])
    assert np.array_equal(a.get("svor"), b.get("svor"))
