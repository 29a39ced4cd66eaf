"""CPU checks of the synthetic workloads' physics."""
import numpy as np
import pytest

from finitevolumesolver_gb300 import workloads


@pytest.mark.parametrize("mach", [1.5, 2.0, 5.0])
def test_shock_state_satisfies_rankine_hugoniot(mach):
    """The post-shock state of the cut-cell workload satisfies the jump
    conditions of a shock moving at S = M c0 into still gas (rho 1, p 1):
    mass, momentum and energy fluxes relative to the shock are continuous."""
    g = workloads.GAMMA
    n = 16
    _, cons = workloads.shock_circles_2d(n, seed=1, mach=mach, x_shock=0.5)
    rho, mx, my, E = (cons[k, 0] for k in range(4))
    post, pre = (0, 0), (0, n - 1)
    r1, r0 = rho[post], rho[pre]
    u1, u0 = mx[post] / r1, mx[pre] / r0
    p1 = (g - 1) * (E[post] - 0.5 * r1 * u1 * u1)
    p0 = (g - 1) * (E[pre] - 0.5 * r0 * u0 * u0)
    assert (r0, u0, p0) == pytest.approx((1.0, 0.0, 1.0), abs=1e-14)
    assert np.all(my == 0.0)
    S = mach * np.sqrt(g * p0 / r0)
    w1, w0 = u1 - S, u0 - S
    mass = (r1 * w1, r0 * w0)
    mom = (r1 * w1 * w1 + p1, r0 * w0 * w0 + p0)
    # total enthalpy flux in the shock frame: rho w (h + w^2/2)
    h1 = g / (g - 1) * p1 / r1
    h0 = g / (g - 1) * p0 / r0
    ener = (r1 * w1 * (h1 + 0.5 * w1 * w1), r0 * w0 * (h0 + 0.5 * w0 * w0))
    for a, b in (mass, mom, ener):
        assert a == pytest.approx(b, rel=1e-13)
    # a compressive shock: denser, faster, higher pressure behind it
    assert r1 > r0 and p1 > p0 and 0 < u1 < S
