"""The sweeps' CFL maximum under the FP32 screen of the exact, fast and
double-float flavours.

A sweep evaluates a face's Einfeldt speed in the flavour's own arithmetic only
where an FP32 estimate plus its error bound reaches the largest speed found so
far, so its maximum must still be the same number as the unscreened one.  The
stable-dt pass computes the same face speeds with the same arithmetic (its
3-D kernel screened the same way, its 1-D and 2-D kernels not): over the same
faces its per-direction dt equals the sweep's level dt bit for bit, for the
exact flavour both equal the oracle's
(DimensionalSplitLevelIntegrator.hpp:240-245 checks exactly this number), and
for the fast and double-float flavours they agree with it to 1e-12.
The states put many faces within rounding of the maximum, carry hypersonic
normal and tangential flow (the cancellations the error bound covers), hold
densities and energies outside the screen's range, or use a gamma outside
(1, 2], where the screen is off."""
import zlib

import numpy as np
import pytest

from finitevolumesolver_gb300 import workloads

pytestmark = pytest.mark.gpu

FLAVOURS = ["fp64_exact", "fp64_fast", "fp64_df"]


def plateau(shape, rank, rng):
    # one uniform state with relative noise 1e-12 and one faster cell: the
    # maximum sits on two faces among thousands within 1e-11 of it
    r = 1.0 + 1e-12 * rng.standard_normal(shape)
    p = 1.0 + 1e-12 * rng.standard_normal(shape)
    vel = [0.3 + 1e-12 * rng.standard_normal(shape) for _ in range(rank)]
    cons = workloads.cons_from_prim(r, vel, p)
    idx = tuple(s // 3 for s in shape)
    cons[(rank + 1,) + idx] *= 1.0 + 1e-9
    return cons


def hypersonic(shape, rank, rng):
    # Mach ~1e3 along x (normal for x sweeps, tangential for the others)
    r = rng.uniform(0.5, 1.5, shape)
    p = rng.uniform(0.5, 1.5, shape)
    vel = [1.2e3 * (1.0 + 0.01 * rng.standard_normal(shape))]
    vel += [rng.uniform(-0.5, 0.5, shape) for _ in range(rank - 1)]
    return workloads.cons_from_prim(r, vel, p)


def hypersonic_mixed(shape, rank, rng):
    # Mach up to ~1e4 in every direction, pressures over six decades
    r = np.exp(rng.uniform(-3, 3, shape))
    p = np.exp(rng.uniform(-7, 7, shape))
    vel = [rng.uniform(-3e3, 3e3, shape) for _ in range(rank)]
    return workloads.cons_from_prim(r, vel, p)


def scaled(shape, rank, rng):
    # densities, momenta and energies times 1e-34 or 1e34 (outside the
    # screen's range) next to ordinary cells of the same velocity and
    # temperature, so the maximum can sit on either kind
    cons = workloads.random_state(shape, rank, seed=int(rng.integers(1 << 30)))
    flat = cons.reshape(rank + 2, -1)
    n = flat.shape[1]
    pick = rng.choice(n, size=(2, max(1, n // 20)), replace=False)
    flat[:, pick[0]] *= 1e-34
    flat[:, pick[1]] *= 1e34
    return cons


def hot_and_light(shape, rank, rng):
    # a few cells with E beyond 2^40 (very hot) and a few light cells (density
    # and momentum times 1e-12, the same pressure: sound 1e6 times faster)
    cons = workloads.random_state(shape, rank, seed=int(rng.integers(1 << 30)))
    flat = cons.reshape(rank + 2, -1)
    n = flat.shape[1]
    pick = rng.choice(n, size=(2, max(1, n // 200)), replace=False)
    flat[rank + 1, pick[0]] *= 1e15
    ke = 0.5 * (flat[1:1 + rank, pick[1]] ** 2).sum(axis=0) / flat[0, pick[1]]
    flat[rank + 1, pick[1]] -= ke * (1.0 - 1e-12)
    flat[:1 + rank, pick[1]] *= 1e-12
    return cons


def cold(shape, rank, rng):
    # nearly pressureless gas: sound speeds ~1e-6, speeds ~1e-3
    r = rng.uniform(0.5, 1.5, shape)
    p = 1e-12 * rng.uniform(0.5, 1.5, shape)
    vel = [1e-3 * rng.uniform(-1, 1, shape) for _ in range(rank)]
    return workloads.cons_from_prim(r, vel, p)


STATES = {"plateau": plateau, "hypersonic": hypersonic, "hypersonic_mixed": hypersonic_mixed,
          "scaled": scaled, "hot_and_light": hot_and_light, "cold": cold}
GRIDS = [(1, [1000]), (2, [150, 41]), (3, [40, 34, 37])]


ORACLE_KIND = {"muscl_hlle": 0, "hllem": 4, "muscl_hllem": 5, "muscl_char": 6, "muscl_prim": 7}


def check_sweeps(fvs, orc, rank, n, cons, prec, gamma=1.4, seg=0, oracle=True,
                 method="muscl_hlle"):
    dx = [0.1, 0.07, 0.05][:rank]
    m = fvs.make_method(flux_method=method, precision=prec, gamma=gamma)
    s = fvs.Solver(n, dx, "periodic", method=m)
    s.set_tiling(seg)
    g = orc.Grid(rank, n, [0] * rank, dx) if oracle else None
    for d in range(rank):
        s.upload(cons)
        ref = s.ComputeStableDt(d)
        assert np.isfinite(ref) and ref > 0
        if g is not None:
            want = g.stable_dt(orc.method(kind=ORACLE_KIND[method]), cons, d, 0)
            if prec == "fp64_exact":
                assert ref == want
            else:
                assert ref == pytest.approx(want, rel=1e-12)
        s.upload(cons)
        level = s.sweep(d, 1e-3 * ref)
        assert level == ref, (d, level, ref)
    s.close()


@pytest.mark.parametrize("prec", FLAVOURS)
@pytest.mark.parametrize("state", sorted(STATES))
@pytest.mark.parametrize("rank,n", GRIDS)
def test_sweep_max_equals_stable_dt(fvs, orc, rank, n, state, prec):
    if state == "scaled" and prec == "fp64_df":
        pytest.skip("double-float has FP32's exponent range: rho u^2 of 1e34 overflows")
    rng = np.random.default_rng(zlib.crc32(f"{rank}{state}".encode()))
    shape = tuple(reversed(n))
    cons = STATES[state](shape, rank, rng)
    cons = cons.reshape([rank + 2] + [1] * (3 - rank) + list(shape))
    check_sweeps(fvs, orc, rank, n, cons, prec)


@pytest.mark.parametrize("seg", [3, 8, 17])
def test_sweep_max_segments(fvs, orc, seg):
    # short segments: the warps' running maxima meet through the sweep's slot
    rng = np.random.default_rng(11)
    n = [40, 34, 37]
    cons = hypersonic_mixed(tuple(reversed(n)), 3, rng)
    for prec in FLAVOURS:
        check_sweeps(fvs, orc, 3, n, cons, prec, seg=seg)


def test_sweep_max_many_blocks(fvs, orc):
    # 96^3: several waves of blocks, later ones start from the published max
    rng = np.random.default_rng(3)
    n = [96, 96, 96]
    cons = workloads.octants_3d(96, seed=4)
    check_sweeps(fvs, orc, 3, n, cons, "fp64_exact")
    check_sweeps(fvs, orc, 3, n, plateau(tuple(reversed(n)), 3, rng), "fp64_exact")
    check_sweeps(fvs, orc, 3, n, hypersonic(tuple(reversed(n)), 3, rng), "fp64_fast",
                 oracle=False)


@pytest.mark.parametrize("gamma", [1.0 + 1e-3, 5.0 / 3.0, 2.0, 2.5, 4.0])
def test_sweep_max_gamma(fvs, orc, gamma):
    # the screen covers 1 < gamma <= 2 and is off above; the oracle's gas has
    # gamma 1.4, so these compare the sweep with the stable-dt pass only
    rng = np.random.default_rng(int(gamma * 1000))
    n = [40, 34, 37]
    shape = tuple(reversed(n))
    r = rng.uniform(0.5, 1.5, shape)
    p = np.exp(rng.uniform(-4, 4, shape))
    vel = [rng.uniform(-50, 50, shape) for _ in range(3)]
    cons = workloads.cons_from_prim(r, vel, p, gamma=gamma)
    for prec in FLAVOURS:
        check_sweeps(fvs, orc, 3, n, cons, prec, gamma=gamma, oracle=False)


@pytest.mark.parametrize("state", ["hypersonic", "plateau", "cold"])
def test_amr_screened_speeds_bit_exact(fvs, orc, state):
    # the AMR patch sweeps and max-speed passes screen their speeds per thread:
    # a three-level hierarchy filled with the state, patch by patch, runs the
    # oracle's dt sequence and state bit for bit (exact FP64)
    h, _ = workloads.amr_blast_2d(64, 3, target=80, sizes=(8, 16))
    rng = np.random.default_rng(zlib.crc32(state.encode()))
    parts = []
    for x0, y0, x1, y1 in h.boxes:
        parts.append(STATES[state]((y1 - y0, x1 - x0), 2, rng).reshape(-1))
    cons = np.concatenate(parts)
    a = fvs.AmrSolver(h)
    a.upload(cons)
    st, dts = a.run(cfl=0.8, t_end=10.0, max_steps=3, log_len=4)
    ref, ref_dts, rs = orc.amr_run(h, cons, 0.8, 10.0, max_steps=3)
    assert st.steps == 3 and st.restarts == rs
    np.testing.assert_array_equal(dts, ref_dts)
    np.testing.assert_array_equal(a.download(), ref)


@pytest.mark.parametrize("prec", ["fp64_exact", "fp64_fast"])
@pytest.mark.parametrize("state", ["hypersonic", "hypersonic_mixed", "plateau", "cold"])
def test_cutcell_screened_speeds(fvs, orc, state, prec):
    # the KBN sweeps screen their CFL speeds over the faces with beta > 0; the
    # stable-dt pass evaluates every such face: same number, bit for bit, and
    # for the exact flavour the oracle's
    n = 100
    circles = [[0.35, 0.4, 0.12], [0.5, 0.45, 0.1], [0.7, 0.7, 0.15]]
    rng = np.random.default_rng(zlib.crc32(f"cc{state}".encode()))
    cons = STATES[state]((n, n), 2, rng).reshape(4, 1, n, n)
    s = fvs.Solver([n, n], [1.0 / n, 1.0 / n], "transmissive",
                   method=fvs.make_method(precision=prec))
    s.set_embedded_circles(circles)
    ref = orc.CutCellGeometry(n, n, circles)
    for d in (0, 1):
        s.upload(cons)
        want = s.ComputeStableDt(d)
        if prec == "fp64_exact":
            assert want == ref.stable_dt(cons, d)
        else:
            assert want == pytest.approx(ref.stable_dt(cons, d), rel=1e-12)
        s.upload(cons)
        level = s.sweep(d, 1e-3 * want)
        assert level == want, (d, level, want)
    s.close()


@pytest.mark.parametrize("method", ["hllem", "muscl_hllem", "muscl_char", "muscl_prim"])
@pytest.mark.parametrize("state", ["hypersonic", "hypersonic_mixed", "plateau", "cold", "scaled"])
def test_hllem_screened_speeds(fvs, orc, method, state):
    # the HLLEM sweeps screen their stable-dt speeds (Roe average over the full
    # velocity, max(c_L, c_R)) with the same bound; exact FP64 only
    rng = np.random.default_rng(zlib.crc32(f"hllem{state}".encode()))
    n = [40, 34, 37]
    cons = STATES[state](tuple(reversed(n)), 3, rng)
    check_sweeps(fvs, orc, 3, n, cons, "fp64_exact", method=method)
