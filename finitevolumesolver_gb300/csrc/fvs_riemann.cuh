// fvs_riemann.cuh -- exact Riemann solver for the perfect gas on the device
// (FP64) and the Godunov flux built on it.
//
// Restates maikel/FiniteVolumeSolver's
//   ExactRiemannSolver<PerfectGas<D>>::ComputeMiddleState
//       src/equations/perfect_gas/ExactRiemannSolver.hpp:34-97
//   NewtonIteration                 include/fub/NewtonIteration.hpp:28-52
//   ExactRiemannSolver::ComputeSignals   ExactRiemannSolver.hpp:105-148
//   ExactRiemannSolver::SolveRiemannProblem (x/t = 0)  ExactRiemannSolver.hpp:204-353
//   Godunov::ComputeNumericFlux / ComputeStableDt
//       include/fub/flux_method/GodunovMethod.hpp:129-183
// with the reference's operation order (the including translation unit is
// compiled with -fmad=false).  The powers of pressure ratios are n-th roots
// (Powers) or CUDA's pow(), and the quotients and square roots of variable
// operands refined reciprocal seeds (Div, Sqrt), so results agree with the
// CPU oracle to ~1e-15 relative rather than bit for bit.
//
// Differences by design:
//  - Newton is bounded by `max_iterations` and never throws: a face that has
//    not met the tolerance keeps its last iterate and is counted as a
//    failure (the reference throws std::runtime_error after 5000 steps).
//  - The start value is selectable: the reference's arithmetic mean, the
//    PVRS/two-rarefaction estimate, or a learned (MLP) estimate, used only
//    where the PVRS/TR start is poor (large residual), that falls back to
//    PVRS/two-rarefaction when non-positive or not finite, or when Newton
//    from it has not converged within 64 steps.
#pragma once

#include "fvs_mlp.cuh"
#include "fvs_physics_exact.cuh"
#include "fvs_physics_fast.cuh"
#include "fvs_roots.cuh"

namespace fvs {
namespace riemann {

enum Guess : int { kGuessMean = 0, kGuessPvrsTr = 1, kGuessMlp = 2 };

struct Options {
  int guess;
  int max_iterations;
  double tol;
  const float* mlp;  // learned-guess parameters (kGuessMlp)
  int root_n;        // RootOrder(gamma): 0, or n with n-th roots in place of pow()
};

// Quotients and square roots of the solver's variable operands: a reciprocal
// (reciprocal square root) seed refined by one third-order step, the fast
// flavour's fast::Math<double> (within ~2 ulp of IEEE), in place of IEEE
// division and sqrt, which cost the FP64 pipe several times as much.
// Operands that are zero, negative, not finite or within 2^2 of the FP64
// range's ends take IEEE division and sqrt, so vacuum and failed states keep
// IEEE semantics (inf, NaN).
__device__ __forceinline__ bool InRange(double b) {
  const unsigned e = static_cast<unsigned>(__double2hiint(b)) & 0x7FFFFFFFu;
  return e >= 0x00200000u && e < 0x7FD00000u;
}
__device__ __forceinline__ double Div(double a, double b) {
  return InRange(b) ? a * fast::Math<double>::Rcp(b) : a / b;
}
__device__ __forceinline__ double Sqrt(double a) {
  return (a > 0.0 && InRange(a)) ? a * fast::Math<double>::Rsqrt(a) : sqrt(a);
}

// PerfectGas::CompleteFromCons and Flux (src/equations/PerfectGas.cpp:52-124)
// with the quotients and square root above: the Godunov sweeps' cell states
// and face flux.
template <int D>
__device__ __forceinline__ void CompleteFromConsFast(const exact::Gas& eq, exact::Complete<D>& q,
                                                     const double* u) {
  q.rho = u[0];
#pragma unroll
  for (int d = 0; d < D; ++d) q.m[d] = u[1 + d];
  q.E = u[1 + D];
  const double e_kin = Div(0.5 * exact::SquaredNorm<D>(q.m), q.rho);
  const double e_int = q.E - e_kin;
  q.p = Div(e_int, eq.gamma_minus_1_inv);
  q.c = Sqrt(Div(eq.gamma * q.p, q.rho));
}

template <int D>
__device__ __forceinline__ void FluxFast(double* f, const exact::Complete<D>& q, int dir) {
  const double velocity = Div(q.m[dir], q.rho);
  f[0] = q.m[dir];
#pragma unroll
  for (int d = 0; d < D; ++d) f[1 + d] = velocity * q.m[d];
  f[1 + dir] += q.p;
  f[1 + D] = velocity * (q.E + q.p);
}

// Scalar-path |m|^2 of the reference's exact solver: (m0^2 + m1^2) + m2^2.
template <int D> __device__ __forceinline__ double SquaredNormScalar(const double* m) {
  if constexpr (D == 1) {
    return m[0] * m[0];
  } else if constexpr (D == 2) {
    return m[0] * m[0] + m[1] * m[1];
  } else {
    return (m[0] * m[0] + m[1] * m[1]) + m[2] * m[2];
  }
}

// PVRS estimate, replaced by the two-rarefaction estimate below min(pL, pR)
// (Toro, Riemann Solvers and Numerical Methods for Fluid Dynamics, 3rd ed.,
// section 9.5); floored at 1e-8 min(pL, pR).
__device__ __forceinline__ double PvrsTrGuess(const Powers& pw, double g, double rhoL, double uL,
                                              double pL, double aL, double rhoR, double uR,
                                              double pR, double aR) {
  const double pmin = pL < pR ? pL : pR;
  const double ppv = 0.5 * (pL + pR) - 0.125 * (uR - uL) * (rhoL + rhoR) * (aL + aR);
  double p0;
  if (ppv >= pmin) {
    p0 = ppv;
  } else {
    const double z = (g - 1.0) / (2.0 * g);
    const double num = aL + aR - 0.5 * (g - 1.0) * (uR - uL);
    const double den = Div(aL, pw.Z(pL, z)) + Div(aR, pw.Z(pR, z));
    p0 = (num > 0.0) ? pw.N(Div(num, den), 1.0 / z) : 0.0;
  }
  const double floor = 1e-8 * pmin;
  return p0 > floor ? p0 : floor;
}

struct SideFn {
  double rho, p, a, A, B;
};

__device__ __forceinline__ double FSide(const SideFn& s, double gm1, double exponent,
                                        const Powers& pw, double q) {
  if (q > s.p) {
    return (q - s.p) * Sqrt(Div(s.A, q + s.B));
  }
  return Div(2.0 * s.a, gm1) * (pw.Z(Div(q, s.p), exponent) - 1.0);
}

__device__ __forceinline__ double DfSide(const SideFn& s, double d_exponent, const Powers& pw,
                                         double q) {
  if (q > s.p) {
    return Sqrt(Div(s.A, s.B + q)) * (1.0 - Div(0.5 * (q - s.p), s.B + q));
  }
  return Div(pw.ZMinus1(Div(q, s.p), d_exponent), s.rho * s.a);
}

// The pressure function's two sides at one pressure: f = fR + fL + du
// (ExactRiemannSolver.hpp:89); the solver's middle velocity reuses fR and fL
// of its final pressure.
struct FEval {
  double x, fR, fL;
};

__device__ __forceinline__ FEval EvalF(const SideFn& L, const SideFn& R, double gm1,
                                       double exponent, const Powers& pw, double x) {
  return FEval{x, FSide(R, gm1, exponent, pw, x), FSide(L, gm1, exponent, pw, x)};
}

// NewtonIteration from the evaluated start e0 (NewtonIteration.hpp:28-52),
// bounded; returns the last evaluation.
__device__ __forceinline__ FEval NewtonFrom(const SideFn& L, const SideFn& R, double du,
                                            double gm1, double exponent, double d_exponent,
                                            const Powers& pw, FEval e0, double tol,
                                            int max_iterations, int& iterations,
                                            int& converged) {
  FEval e = e0;
  double fx = e.fR + e.fL + du;
  int counter = 0;
  double err = fabs(fx);
  while (err > tol && counter < max_iterations) {
    const double x = e.x;
    const double dfx = DfSide(R, d_exponent, pw, x) + DfSide(L, d_exponent, pw, x);
    const double offset = Div(fx, dfx);
    const double next = x - offset;
    e = EvalF(L, R, gm1, exponent, pw,
              ((next - next) != (next - next) || next < 0.0) ? 0.5 * x : next);
    fx = e.fR + e.fL + du;
    err = fabs(fx);
    counter += 1;
  }
  iterations = counter;
  converged = !(err > tol);
  return e;
}

template <int D>
__device__ __forceinline__ Star ComputeMiddleState(const exact::Gas& eq,
                                                   const exact::Complete<D>& left,
                                                   const exact::Complete<D>& right, int dir,
                                                   const Options& opt) {
  const double g = eq.gamma;
  const double gp1 = g + 1.0;
  const double gm1 = g - 1.0;
  SideFn L, R;
  L.rho = left.rho;
  L.p = left.p;
  L.a = left.c;
  L.A = Div(2.0, gp1 * L.rho);
  L.B = gm1 / gp1 * L.p;
  R.rho = right.rho;
  R.p = right.p;
  R.a = right.c;
  R.A = Div(2.0, gp1 * R.rho);
  R.B = gm1 / gp1 * R.p;
  const double exponent = 0.5 * gm1 / g;
  const double d_exponent = -0.5 * gp1 / g;
  const Powers pw(opt.root_n);
  const double uL = Div(left.m[dir], left.rho);
  const double uR = Div(right.m[dir], right.rho);
  const double du = uR - uL;
  Star st;
  st.fallback = 0;
  double x0;
  if (opt.guess == kGuessMean) {
    x0 = 0.5 * (L.p + R.p);
  } else {
    const double pv = PvrsTrGuess(pw, g, L.rho, uL, L.p, L.a, R.rho, uR, R.p, R.a);
    x0 = pv;
    // Cost-aware use of the learned start: the network costs about one
    // Newton step (its 5-64-64-1 FP32 multiply-adds against two FP64 roots
    // or pow evaluations per step), so it is used only where it is expected to
    // save at least one step.  Newton converges quadratically, so from a
    // start whose relative residual is r = |f(p0)| / (aL + aR) it needs
    // about k(r) = ceil(log2(log(tol') / log(r))) steps to reach
    // |f| <= tol, tol' = tol / (aL + aR).  The PVRS/TR start's r is known
    // from its residual; the learned start's is taken as kLearnedRelErr,
    // the network's typical relative error in p*.  Weak waves (most faces of
    // a real flow), where PVRS/TR is accurate to second order in the wave
    // strength, keep their start and never pay for the network.
    constexpr float kLearnedRelErr = 0.01f;
    double f_pv = 0.0;
    FEval e_pv{pv, 0.0, 0.0};
    bool screened = false;
    if (opt.guess == kGuessMlp) {
      e_pv = EvalF(L, R, gm1, exponent, pw, pv);
      f_pv = e_pv.fR + e_pv.fL + du;
      const float scale = static_cast<float>(L.a + R.a);
      const float lt = __log2f(static_cast<float>(opt.tol) / scale);  // < 0 for tol < scale
      auto steps = [&](float r) -> float {
        if (!(r > exp2f(lt))) return 0.0f;   // already within the tolerance
        if (!(r < 0.5f)) return 1e30f;       // outside the quadratic regime
        return ceilf(__log2f(lt / __log2f(r)));
      };
      const float r_pv = static_cast<float>(fabs(f_pv)) / scale;
      screened = !(steps(r_pv) >= steps(kLearnedRelErr) + 1.0f);
      if (screened || !opt.mlp) {
        // PVRS/TR start, reusing the residual just evaluated
        const FEval e = NewtonFrom(L, R, du, gm1, exponent, d_exponent, pw, e_pv, opt.tol,
                                   opt.max_iterations, st.iterations, st.converged);
        st.p = e.x;
        st.u = 0.5 * (uL + uR) + 0.5 * (e.fR - e.fL);
        return st;
      }
    }
    if (opt.guess == kGuessMlp && opt.mlp && !screened) {
      const double learned = mlp::GuessStarPressure(opt.mlp, L.rho, uL, L.p, L.a, R.rho, uR,
                                                    R.p, R.a);
      if (learned > 0.0 && learned < 1.7976931348623157e308) {
        x0 = learned;
      } else {
        st.fallback = 1;
      }
    }
    if (opt.guess == kGuessMlp && !st.fallback) {
      int it, ok;
      // a learned start gets at most 64 steps before the PVRS/TR restart
      const int learned_max = opt.max_iterations < 64 ? opt.max_iterations : 64;
      FEval e = NewtonFrom(L, R, du, gm1, exponent, d_exponent, pw,
                           EvalF(L, R, gm1, exponent, pw, x0), opt.tol, learned_max, it, ok);
      if (!ok) {
        // the learned start did not converge within the bound: fall back
        st.fallback = 1;
        int it2, ok2;
        e = NewtonFrom(L, R, du, gm1, exponent, d_exponent, pw, e_pv, opt.tol,
                       opt.max_iterations, it2, ok2);
        it += it2;
        ok = ok2;
      }
      st.p = e.x;
      st.iterations = it;
      st.converged = ok;
      st.u = 0.5 * (uL + uR) + 0.5 * (e.fR - e.fL);
      return st;
    }
  }
  const FEval e = NewtonFrom(L, R, du, gm1, exponent, d_exponent, pw,
                             EvalF(L, R, gm1, exponent, pw, x0), opt.tol, opt.max_iterations,
                             st.iterations, st.converged);
  st.p = e.x;
  st.u = 0.5 * (uL + uR) + 0.5 * (e.fR - e.fL);
  return st;
}

// max(0, |s0|, |s1|) with the exact solver's signal speeds
// (ExactRiemannSolver.hpp:105-148, GodunovMethod.hpp:173-183).
template <int D>
__device__ __forceinline__ double SignalMaxSpeed(const exact::Gas& eq,
                                                 const exact::Complete<D>& left,
                                                 const exact::Complete<D>& right, int dir,
                                                 double pM) {
  const double g = eq.gamma;
  const double gp1 = g + 1.0;
  const double gm1 = g - 1.0;
  const double uL = Div(left.m[dir], left.rho);
  const double aL = left.c;
  const double pL = left.p;
  const double pL_ratio = Div(pM, pL);
  double s0, s1;
  if (pM > pL) {
    s0 = uL - aL * Sqrt(Div(gp1 * pL_ratio + gm1, 2.0 * g));
  } else {
    s0 = uL - aL;
  }
  const double uR = Div(right.m[dir], right.rho);
  const double aR = right.c;
  const double pR = right.p;
  const double pR_ratio = Div(pM, pR);
  if (pM > pR) {
    s1 = uR + aR * Sqrt(Div(gp1 * pR_ratio + gm1, 2.0 * g));
  } else {
    s1 = uR + aR;
  }
  double s = 0.0;
  const double a0 = fabs(s0), a1 = fabs(s1);
  s = (s < a0) ? a0 : s;  // std::max(x, |y|)
  s = (s < a1) ? a1 : s;
  return s;
}

// SolveRiemannProblem sampled at x/t = 0 (ExactRiemannSolver.hpp:204-353).
template <int D>
__device__ __forceinline__ void Sample(const exact::Gas& eq, exact::Complete<D>& state,
                                       const exact::Complete<D>& left,
                                       const exact::Complete<D>& right, int dir, double pM,
                                       double uM, const Options& opt) {
  const Powers pw(opt.root_n);
  const double g = eq.gamma;
  const double gp1 = g + 1.0;
  const double gm1 = g - 1.0;
  auto set_momentum = [dir](exact::Complete<D>& s, double momentum,
                            const exact::Complete<D>& side) {
    if constexpr (D == 1) {
      s.m[0] = momentum;
    } else {
#pragma unroll
      for (int d = 0; d < D; ++d) s.m[d] = s.rho * Div(side.m[d], side.rho);
      s.m[dir] = momentum;
    }
  };
  auto from_prim = [&eq](exact::Complete<D>& s) {
    const double rhoE_kin = Div(0.5 * SquaredNormScalar<D>(s.m), s.rho);
    const double rhoE_internal = s.p * eq.gamma_minus_1_inv;
    s.E = rhoE_internal + rhoE_kin;
    s.c = Sqrt(Div(eq.gamma * s.p, s.rho));
  };
  if (0.0 <= uM) {
    const double uL = Div(left.m[dir], left.rho);
    const double aL = left.c;
    const double pL = left.p;
    const double p_ratio = Div(pM, pL);
    const double g_ratio = gm1 / gp1;
    if (pM > pL) {
      const double shock_speed = uL - aL * Sqrt(Div(gp1 * p_ratio + gm1, 2.0 * g));
      if (shock_speed < 0.0) {
        state.rho = Div(left.rho * (p_ratio + g_ratio), g_ratio * p_ratio + 1.0);
        set_momentum(state, state.rho * uM, left);
        state.p = pM;
        from_prim(state);
      } else {
        state = left;
      }
    } else {
      const double aM = aL * pw.Z(p_ratio, gm1 / (2.0 * g));
      const double shock_speed_TL = uM - aM;
      const double shock_speed_HL = uL - aL;
      if (0.0 < shock_speed_HL) {
        state = left;
      } else if (shock_speed_TL < 0.0) {
        state.rho = left.rho * pw.InvGamma(p_ratio, 1 / g);
        set_momentum(state, state.rho * uM, left);
        state.p = pM;
        from_prim(state);
      } else {
        state.rho = left.rho * pw.N2(2.0 / gp1 + Div(g_ratio * uL, aL), 2.0 / gm1);
        const double u = 2.0 / gp1 * (aL + 0.5 * gm1 * uL);
        set_momentum(state, state.rho * u, left);
        state.p = pL * pw.N(2.0 / gp1 + Div(g_ratio * uL, aL), 2.0 * g / gm1);
        from_prim(state);
      }
    }
  } else {
    const double uR = Div(right.m[dir], right.rho);
    const double aR = right.c;
    const double pR = right.p;
    const double p_ratio = Div(pM, pR);
    const double g_ratio = gm1 / gp1;
    if (pM > pR) {
      const double shock_speed = uR + aR * Sqrt(Div(gp1 * p_ratio + gm1, 2.0 * g));
      if (0.0 < shock_speed) {
        state.rho = Div(right.rho * (p_ratio + g_ratio), g_ratio * p_ratio + 1.0);
        set_momentum(state, state.rho * uM, right);
        state.p = pM;
        from_prim(state);
      } else {
        state = right;
      }
    } else {
      const double aM = aR * pw.Z(p_ratio, gm1 / (2.0 * g));
      const double shock_speed_TR = uM + aM;
      const double shock_speed_HR = uR + aR;
      if (shock_speed_HR <= 0.0) {
        state = right;
      } else if (shock_speed_TR >= 0.0) {
        state.rho = right.rho * pw.InvGamma(p_ratio, 1 / g);
        set_momentum(state, state.rho * uM, right);
        state.p = pM;
        from_prim(state);
      } else {
        state.rho = right.rho * pw.N2(2.0 / gp1 - Div(g_ratio * uR, aR), 2.0 / gm1);
        const double u = 2.0 / gp1 * (-aR + 0.5 * gm1 * uR);
        set_momentum(state, state.rho * u, right);
        state.p = pR * pw.N(2.0 / gp1 - Div(g_ratio * uR, aR), 2.0 * g / gm1);
        from_prim(state);
      }
    }
  }
}

// Godunov flux: the physical flux of the exact solution at x/t = 0
// (GodunovMethod.hpp:129-135).  Faces with a non-positive density keep the
// left state (the reference leaves the solution untouched there).
template <int D>
__device__ __forceinline__ Star GodunovFlux(const exact::Gas& eq, double* nf,
                                            const exact::Complete<D>& L,
                                            const exact::Complete<D>& R, int dir,
                                            const Options& opt) {
  exact::Complete<D> sol = L;
  Star st{0.0, 0.0, 0, 1, 0};
  if (0.0 < L.rho && 0.0 < R.rho) {
    st = ComputeMiddleState<D>(eq, L, R, dir, opt);
    Sample<D>(eq, sol, L, R, dir, st.p, st.u, opt);
  }
  FluxFast<D>(nf, sol, dir);
  return st;
}

}  // namespace riemann
}  // namespace fvs
