"""The error bound behind the FP32 screen of the CFL speeds (fvs_sweep.cuh,
FilteredCfl: the Einfeldt speed and the HLLEM stable-dt speed), checked on
the CPU.

The sweeps skip a face's FP64 Einfeldt speed s when its FP32 estimate s32
satisfies s32 / 1024 + sqrt(max(h_L, h_R)) / 64 + 2^-24 + s32 < threshold,
which is safe if |s - s32| never exceeds that bound.  This test emulates the
kernel's FP32 arithmetic in numpy: every FP32 operation rounds to FP32, the
approximate reciprocal and reciprocal square root get a random error of up to
2^-22 (their documented 2-ulp bound), and the states are converted from the
FP64 cells.  The FP64 speed follows the exact flavour's formulas.  States
cover the bound's domain (2^-30 <= rho <= 2^30, |m| <= 2^30, |E| <= 2^40,
positive FP32 pressure) with Mach numbers up to 3e4, normal and tangential,
near-sonic faces, near-vacuum pressures and density jumps of 10^6, for gammas
in (1, 2]."""
import zlib

import numpy as np
import pytest

F32 = np.float32


def r32(x):
    return np.asarray(x, dtype=np.float64).astype(F32)


def fma32(a, b, c):
    # FP32 fused multiply-add: the product is exact in FP64, one rounding
    return r32(a.astype(np.float64) * b.astype(np.float64) + c.astype(np.float64))


def approx(x, rng):
    # an approximate FP32 unit: within 2^-22 relative of the exact value
    e = rng.uniform(-1.0, 1.0, x.shape) * 2.0 ** -22
    return r32(x.astype(np.float64) * (1.0 + e))


def wave32(u, d, g, rng):
    """fast::MakeWave<D, float> (fvs_physics_fast.cuh) in emulated FP32."""
    rho, m, E = u[0], u[1:-1], u[-1]
    rs = approx(1.0 / np.sqrt(rho.astype(np.float64)), rng)  # rsqrtf
    ir = r32(rs * rs)
    sq = r32(rho * rs)
    sn = r32(m[0] * m[0])
    for k in range(1, m.shape[0]):
        sn = fma32(m[k], m[k], sn)
    ke = r32(r32(F32(0.5) * sn) * ir)
    p = r32(r32(E - ke) * F32(g - 1.0))
    un = r32(m[d] * ir)
    h = r32(r32(E + p) * ir)
    x = r32(r32(F32(g) * p) * ir)
    xs = np.where(x > 0, x, F32(1))
    a = np.where(x > 0, r32(x * approx(1.0 / np.sqrt(xs.astype(np.float64)), rng)), F32(0))
    return sq, un, h, a, p


def speed32(L, R, g, rng):
    """fast::FaceMaxSpeed<float>."""
    sqL, uL, hL, aL, _ = L
    sqR, uR, hR, aR, _ = R
    oo = approx(1.0 / (r32(sqL + sqR)).astype(np.float64), rng)  # __fdividef(1, x)
    roeU = r32(fma32(uL, sqL, r32(uR * sqR)) * oo)
    roeH = r32(fma32(hL, sqL, r32(hR * sqR)) * oo)
    x = r32(F32(g - 1.0) * fma32(r32(F32(-0.5) * roeU), roeU, roeH))
    xs = np.where(x > 0, x, F32(1))
    roeA = np.where(x > 0, r32(x * approx(1.0 / np.sqrt(xs.astype(np.float64)), rng)), F32(0))
    sL = np.minimum(r32(uL - aL), r32(roeU - roeA))
    sR = np.maximum(r32(roeU + roeA), r32(uR + aR))
    return np.maximum(np.maximum(F32(0), np.abs(sL)), np.abs(sR))


def speed32_hllem(cL, cR, d, g, rng):
    """HllemScreen::Speed (fvs_sweep.cuh) in emulated FP32, from the cells."""
    def wave(c):
        rho, m, E = c[0], c[1:-1], c[-1]
        rs = approx(1.0 / np.sqrt(rho.astype(np.float64)), rng)
        ir = r32(rs * rs)
        sq = r32(rho * rs)
        u = [r32(m[k] * ir) for k in range(m.shape[0])]
        sn = r32(m[0] * m[0])
        for k in range(1, m.shape[0]):
            sn = fma32(m[k], m[k], sn)
        ke = r32(r32(F32(0.5) * sn) * ir)
        p = r32(r32(E - ke) * F32(g - 1.0))
        h = r32(r32(E + p) * ir)
        x = r32(r32(F32(g) * p) * ir)
        xs = np.where(x > 0, x, F32(1))
        a = np.where(x > 0, r32(x * approx(1.0 / np.sqrt(xs.astype(np.float64)), rng)), F32(0))
        return sq, u, h, a
    sqL, uL, hL, aL = wave(cL)
    sqR, uR, hR, aR = wave(cR)
    oo = approx(1.0 / (r32(sqL + sqR)).astype(np.float64), rng)
    wL, wR = r32(sqL * oo), r32(sqR * oo)
    roeU = [fma32(wL, uL[k], r32(wR * uR[k])) for k in range(len(uL))]
    sqN = np.zeros_like(wL)
    for k in range(len(roeU)):
        sqN = fma32(roeU[k], roeU[k], sqN)
    roeH = fma32(wL, hL, r32(wR * hR))
    x = r32(F32(g - 1.0) * fma32(np.full_like(sqN, F32(-0.5)), sqN, roeH))
    xs = np.where(x > 0, x, F32(1))
    roeA = np.where(x > 0, r32(x * approx(1.0 / np.sqrt(xs.astype(np.float64)), rng)), F32(0))
    maxA = np.maximum(aL, aR)
    sL = np.minimum(r32(uL[d] - maxA), r32(roeU[d] - roeA))
    sR = np.maximum(r32(roeU[d] + roeA), r32(uR[d] + maxA))
    return np.maximum(np.abs(sL), np.abs(sR)), (aL > 0) & (aR > 0), np.maximum(hL, hR)


def speed64_hllem(uL, uR, d, g):
    """HllemMaxSpeed of the exact flavour (fvs_hllem.cuh)."""
    def comp(u):
        rho, m, E = u[0], u[1:-1], u[-1]
        p = (E - 0.5 * (m * m).sum(axis=0) / rho) / (1.0 / (g - 1.0))
        return rho, m / rho, (E + p) / rho, np.sqrt(g * p / rho)
    rL, vL, hL, aL = comp(uL)
    rR, vR, hR, aR = comp(uR)
    sqL, sqR = np.sqrt(rL), np.sqrt(rR)
    wL, wR = sqL / (sqL + sqR), sqR / (sqL + sqR)
    roeU = wL * vL + wR * vR
    roeH = wL * hL + wR * hR
    roeA = np.sqrt((g - 1.0) * (roeH - 0.5 * (roeU * roeU).sum(axis=0)))
    maxA = np.maximum(aL, aR)
    sL = np.minimum(vL[d] - maxA, roeU[d] - roeA)
    sR = np.maximum(roeU[d] + roeA, vR[d] + maxA)
    return np.maximum(np.abs(sL), np.abs(sR))


def speed64(uL, uR, d, g):
    """The exact flavour's Einfeldt face speed (fvs_physics_exact.cuh)."""
    def comp(u):
        rho, m, E = u[0], u[1:-1], u[-1]
        p = (E - 0.5 * (m * m).sum(axis=0) / rho) / (1.0 / (g - 1.0))
        return rho, m[d] / rho, (E + p) / rho, np.sqrt(g * p / rho)
    rL, vL, hL, aL = comp(uL)
    rR, vR, hR, aR = comp(uR)
    sqL, sqR = np.sqrt(rL), np.sqrt(rR)
    roeU = (vL * sqL + vR * sqR) / (sqL + sqR)
    roeH = (hL * sqL + hR * sqR) / (sqL + sqR)
    roeA = np.sqrt((g - 1.0) * (roeH - 0.5 * roeU * roeU))
    sL = np.minimum(vL - aL, roeU - roeA)
    sR = np.maximum(roeU + roeA, vR + aR)
    return np.maximum(np.maximum(0.0, np.abs(sL)), np.abs(sR))


def states(rng, n, dim, g, kind):
    lrho = rng.uniform(-20, 20, n) * np.log(2.0)
    rho = np.exp(lrho)
    if kind == "jump":  # density ratios up to 1e6 between the two cells
        rho = rho * np.exp(rng.uniform(-7, 7, n))
    c0 = np.exp(rng.uniform(-6, 6, n))  # sound speed scale
    p = rho * c0 * c0 / g
    if kind == "vacuum":
        p = p * np.exp(rng.uniform(-25, 0, n))
    mach = {"subsonic": 0.9, "hyper": 3e4, "jump": 30.0, "vacuum": 10.0, "sonic": 1.0}[kind]
    vel = rng.normal(size=(dim, n))
    vel = vel / np.linalg.norm(vel, axis=0) * c0 * rng.uniform(0, mach, n)
    if kind == "sonic":  # normal velocity close to +-c
        vel[0] = c0 * rng.choice([-1.0, 1.0], n) * (1.0 + rng.uniform(-1e-3, 1e-3, n))
    E = p / (g - 1.0) + 0.5 * rho * (vel * vel).sum(axis=0)
    return np.concatenate([rho[None], rho * vel, E[None]])


@pytest.mark.parametrize("speed", ["einfeldt", "hllem"])
@pytest.mark.parametrize("gamma", [1.0 + 1e-3, 1.4, 5.0 / 3.0, 2.0])
@pytest.mark.parametrize("kind", ["subsonic", "sonic", "hyper", "jump", "vacuum"])
def test_screen_bound_holds(gamma, kind, speed):
    rng = np.random.default_rng(zlib.crc32(f"{gamma:.6f}{kind}{speed}".encode()))
    n, dim = 200_000, 3
    uL = states(rng, n, dim, gamma, kind)
    uR = states(rng, n, dim, gamma, kind)
    if kind in ("subsonic", "sonic"):  # neighbours: small perturbations of the left state
        uR = uL * (1.0 + rng.uniform(-0.05, 0.05, uL.shape))
        uR[-1] = np.maximum(uR[-1], 0.5 * (uR[1:-1] ** 2).sum(axis=0) / uR[0] * 1.0001)
    for d in range(dim):
        cL, cR = r32(uL), r32(uR)
        ok = np.ones(n, bool)
        for c in (cL, cR):
            ok &= (c[0] >= 2.0 ** -30) & (c[0] <= 2.0 ** 30) & (np.abs(c[-1]) <= 2.0 ** 40)
            ok &= (np.abs(c[1:-1]) <= 2.0 ** 30).all(axis=0)
        with np.errstate(all="ignore"):
            if speed == "einfeldt":
                wl = wave32(cL, d, gamma, rng)
                wr = wave32(cR, d, gamma, rng)
                ok &= (wl[3] > 0) & (wr[3] > 0)
                s32 = speed32(wl, wr, gamma, rng).astype(np.float64)
                s64 = speed64(uL, uR, d, gamma)
                hmax = np.maximum(wl[2], wr[2])
            else:
                s32, pos, hmax = speed32_hllem(cL, cR, d, gamma, rng)
                ok &= pos
                s32 = s32.astype(np.float64)
                s64 = speed64_hllem(uL, uR, d, gamma)
        sh = np.sqrt(hmax.astype(np.float64))
        bound = s32 / 1024.0 + sh / 64.0 + 2.0 ** -24
        sel = ok & np.isfinite(s64)
        assert sel.sum() > n // 20  # hypersonic states often leave the domain
        err = np.abs(s64[sel] - s32[sel])
        worst = float((err / bound[sel]).max())
        assert worst < 0.5, (kind, gamma, d, worst)
