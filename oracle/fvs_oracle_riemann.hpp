// fvs_oracle_riemann.hpp -- CPU oracle: exact Riemann solver for the perfect
// gas and the Godunov flux built on it.
//
// TEST INFRASTRUCTURE ONLY (see fvs_oracle.hpp).  Follows
//   src/equations/perfect_gas/ExactRiemannSolver.hpp:34-353
//   include/fub/NewtonIteration.hpp:28-52
//   include/fub/flux_method/GodunovMethod.hpp:129-199
// The Newton start value and tolerance are parameters: the reference uses
// the arithmetic mean 0.5*(pL+pR) and |f(p)| <= 1e-7 (kGuessMean, tol 1e-7).
#pragma once

#include "fvs_oracle.hpp"

namespace fvs_oracle {

// Scalar-path |m|^2: the reference's exact solver works on contiguous
// Eigen::Array<double, Dim, 1> vectors, whose squaredNorm() is evaluated with
// one SSE2 packet for the first two components: (m0^2 + m1^2) + m2^2.
template <int D> inline double SquaredNormScalar(const double* m) {
  if constexpr (D == 1) {
    return m[0] * m[0];
  } else if constexpr (D == 2) {
    return m[0] * m[0] + m[1] * m[1];
  } else {
    return (m[0] * m[0] + m[1] * m[1]) + m[2] * m[2];
  }
}

enum Guess : int { kGuessMean = 0, kGuessPvrsTr = 1, kGuessGiven = 2 };

struct NewtonResult {
  double p;
  int iterations;
  int converged;  // 0 when max_iterations was reached with |f| > tol
};

struct StarState {
  double pM;
  double uM;
  int iterations;
  int converged;
};

// Newton-Raphson for the star pressure  include/fub/NewtonIteration.hpp:28-52.
// A non-finite or negative iterate is replaced by half the previous one.
template <typename F, typename DF>
inline NewtonResult NewtonIteration(F&& f, DF&& df, double x0, double tol,
                                    int max_iterations) {
  double x = x0;
  double fx = f(x);
  int counter = 0;
  double err = std::abs(fx);
  while (err > tol && counter < max_iterations) {
    const double dfx = df(x);
    const double offset = fx / dfx;
    const double next = x - offset;
    x = ((next - next) != (next - next) || next < 0.0) ? 0.5 * x : next;
    fx = f(x);
    err = std::abs(fx);
    counter += 1;
  }
  NewtonResult r;
  r.p = x;
  r.iterations = counter;
  r.converged = !(counter == max_iterations && err > tol);
  return r;
}

// Primitive-variable (PVRS) guess, replaced by the two-rarefaction guess when
// it falls below min(pL, pR) (Toro, "Riemann Solvers and Numerical Methods
// for Fluid Dynamics", 3rd ed., section 9.5).  Not a reference behaviour.
inline double PvrsTrGuess(const Gas& eq, double rhoL, double uL, double pL,
                          double aL, double rhoR, double uR, double pR,
                          double aR) {
  const double g = eq.gamma;
  const double pmin = std::min(pL, pR);
  const double ppv =
      0.5 * (pL + pR) - 0.125 * (uR - uL) * (rhoL + rhoR) * (aL + aR);
  double p0;
  if (ppv >= pmin) {
    p0 = ppv;
  } else {
    const double z = (g - 1.0) / (2.0 * g);
    const double num = aL + aR - 0.5 * (g - 1.0) * (uR - uL);
    const double den = aL / std::pow(pL, z) + aR / std::pow(pR, z);
    p0 = (num > 0.0) ? std::pow(num / den, 1.0 / z) : 0.0;
  }
  const double floor = 1e-8 * pmin;
  return p0 > floor ? p0 : floor;
}

// ExactRiemannSolver<PerfectGas<D>>::ComputeMiddleState
// src/equations/perfect_gas/ExactRiemannSolver.hpp:34-97.
template <int D>
inline StarState ComputeMiddleState(const Gas& eq, const Complete<D>& left,
                                    const Complete<D>& right, int dir,
                                    int guess, double given_guess, double tol,
                                    int max_iterations) {
  const double g = eq.gamma;
  const double gp1 = g + 1.0;
  const double gm1 = g - 1.0;
  const double rhoL = left.rho;
  const double pL = left.p;
  const double aL = left.c;
  const double A_l = 2.0 / (gp1 * rhoL);
  const double B_l = gm1 / gp1 * pL;
  const double exponent = 0.5 * gm1 / g;
  const double d_exponent = -0.5 * gp1 / g;
  auto f_left = [=](double p) {
    if (p > pL) {
      return (p - pL) * std::sqrt(A_l / (p + B_l));
    } else {
      return 2.0 * aL / gm1 * (std::pow(p / pL, exponent) - 1.0);
    }
  };
  auto df_left = [=](double p) {
    if (p > pL) {
      return std::sqrt(A_l / (B_l + p)) * (1.0 - 0.5 * (p - pL) / (B_l + p));
    } else {
      return std::pow(p / pL, d_exponent) / (rhoL * aL);
    }
  };
  const double rhoR = right.rho;
  const double pR = right.p;
  const double aR = right.c;
  const double A_r = 2.0 / (gp1 * rhoR);
  const double B_r = gm1 / gp1 * pR;
  auto f_right = [=](double p) {
    if (p > pR) {
      return (p - pR) * std::sqrt(A_r / (p + B_r));
    } else {
      return 2 * aR / gm1 * (std::pow(p / pR, exponent) - 1.0);
    }
  };
  auto df_right = [=](double p) {
    if (p > pR) {
      return std::sqrt(A_r / (B_r + p)) * (1.0 - 0.5 * (p - pR) / (B_r + p));
    } else {
      return std::pow(p / pR, d_exponent) / (rhoR * aR);
    }
  };
  const double uL = left.m[dir] / left.rho;
  const double uR = right.m[dir] / right.rho;
  const double du = uR - uL;
  auto f = [=](double h) { return f_right(h) + f_left(h) + du; };
  auto df = [=](double h) { return df_right(h) + df_left(h); };
  double x0 = 0.5 * (pL + pR);
  if (guess == kGuessPvrsTr) {
    x0 = PvrsTrGuess(eq, rhoL, uL, pL, aL, rhoR, uR, pR, aR);
  } else if (guess == kGuessGiven) {
    x0 = given_guess;
  }
  const NewtonResult nr = NewtonIteration(f, df, x0, tol, max_iterations);
  const double pM = nr.p;
  const double fL = f_left(pM);
  const double fR = f_right(pM);
  const double uM = 0.5 * (uL + uR) + 0.5 * (fR - fL);
  return StarState{pM, uM, nr.iterations, nr.converged};
}

// ExactRiemannSolver::ComputeSignals
// src/equations/perfect_gas/ExactRiemannSolver.hpp:105-148.
template <int D>
inline void ExactSignals(const Gas& eq, const Complete<D>& left,
                         const Complete<D>& right, int dir, double pM,
                         double& s0, double& s1) {
  const double g = eq.gamma;
  const double gp1 = g + 1.0;
  const double gm1 = g - 1.0;
  const double uL = left.m[dir] / left.rho;
  const double aL = left.c;
  const double pL = left.p;
  const double pL_ratio = pM / pL;
  if (pM > pL) {
    s0 = uL - aL * std::sqrt((gp1 * pL_ratio + gm1) / (2.0 * g));
  } else {
    s0 = uL - aL;
  }
  const double uR = right.m[dir] / right.rho;
  const double aR = right.c;
  const double pR = right.p;
  const double pR_ratio = pM / pR;
  if (pM > pR) {
    s1 = uR + aR * std::sqrt((gp1 * pR_ratio + gm1) / (2.0 * g));
  } else {
    s1 = uR + aR;
  }
}

// ExactRiemannSolver::SolveRiemannProblem sampled at x/t = 0
// src/equations/perfect_gas/ExactRiemannSolver.hpp:204-353.  Given (pM, uM).
template <int D>
inline void SampleRiemann(const Gas& eq, Complete<D>& state,
                          const Complete<D>& left, const Complete<D>& right,
                          int dir, double pM, double uM) {
  auto set_momentum = [dir](Complete<D>& s, double momentum,
                            const Complete<D>& side) {
    if constexpr (D == 1) {
      s.m[0] = momentum;
    } else {
      for (int d = 0; d < D; ++d) s.m[d] = s.rho * (side.m[d] / side.rho);
      s.m[dir] = momentum;
    }
  };
  auto from_prim = [&eq](Complete<D>& s) {
    const double rhoE_kin = 0.5 * SquaredNormScalar<D>(s.m) / s.rho;
    const double rhoE_internal = s.p * eq.gamma_minus_1_inv;
    s.E = rhoE_internal + rhoE_kin;
    s.c = std::sqrt(eq.gamma * s.p / s.rho);
  };
  const double g = eq.gamma;
  const double gp1 = g + 1.0;
  const double gm1 = g - 1.0;
  if (0.0 <= uM) {
    const double uL = left.m[dir] / left.rho;
    const double aL = left.c;
    const double pL = left.p;
    const double p_ratio = pM / pL;
    const double g_ratio = gm1 / gp1;
    if (pM > pL) {
      const double shock_speed =
          uL - aL * std::sqrt((gp1 * p_ratio + gm1) / (2.0 * g));
      if (shock_speed < 0.0) {
        state.rho = left.rho * (p_ratio + g_ratio) / (g_ratio * p_ratio + 1.0);
        set_momentum(state, state.rho * uM, left);
        state.p = pM;
        from_prim(state);
      } else {
        state = left;
      }
    } else {
      const double aM = aL * std::pow(p_ratio, gm1 / (2.0 * g));
      const double shock_speed_TL = uM - aM;
      const double shock_speed_HL = uL - aL;
      if (0.0 < shock_speed_HL) {
        state = left;
      } else if (shock_speed_TL < 0.0) {
        state.rho = left.rho * std::pow(p_ratio, 1 / g);
        set_momentum(state, state.rho * uM, left);
        state.p = pM;
        from_prim(state);
      } else {
        state.rho =
            left.rho * std::pow(2.0 / gp1 + g_ratio * uL / aL, 2.0 / gm1);
        const double u = 2.0 / gp1 * (aL + 0.5 * gm1 * uL);
        set_momentum(state, state.rho * u, left);
        state.p = pL * std::pow(2.0 / gp1 + g_ratio * uL / aL, 2.0 * g / gm1);
        from_prim(state);
      }
    }
  } else {
    const double uR = right.m[dir] / right.rho;
    const double aR = right.c;
    const double pR = right.p;
    const double p_ratio = pM / pR;
    const double g_ratio = gm1 / gp1;
    if (pM > pR) {
      const double shock_speed =
          uR + aR * std::sqrt((gp1 * p_ratio + gm1) / (2.0 * g));
      if (0.0 < shock_speed) {
        state.rho =
            right.rho * (p_ratio + g_ratio) / (g_ratio * p_ratio + 1.0);
        set_momentum(state, state.rho * uM, right);
        state.p = pM;
        from_prim(state);
      } else {
        state = right;
      }
    } else {
      const double aM = aR * std::pow(p_ratio, gm1 / (2.0 * g));
      const double shock_speed_TR = uM + aM;
      const double shock_speed_HR = uR + aR;
      if (shock_speed_HR <= 0.0) {
        state = right;
      } else if (shock_speed_TR >= 0.0) {
        state.rho = right.rho * std::pow(p_ratio, 1 / g);
        set_momentum(state, state.rho * uM, right);
        state.p = pM;
        from_prim(state);
      } else {
        state.rho =
            right.rho * std::pow(2.0 / gp1 - g_ratio * uR / aR, 2.0 / gm1);
        const double u = 2.0 / gp1 * (-aR + 0.5 * gm1 * uR);
        set_momentum(state, state.rho * u, right);
        state.p =
            pR * std::pow(2.0 / gp1 - g_ratio * uR / aR, 2.0 * g / gm1);
        from_prim(state);
      }
    }
  }
}

struct ExactOptions {
  int guess = kGuessMean;
  double tol = 1e-7;
  int max_iterations = 5000;
};

// Godunov<PerfectGas<D>, ExactRiemannSolver>::ComputeNumericFlux
// include/fub/flux_method/GodunovMethod.hpp:129-135.  Returns the Newton
// iteration count; *converged reports whether Newton met the tolerance.
template <int D>
inline int GodunovFlux(const Gas& eq, double* nf, const Complete<D>& L,
                       const Complete<D>& R, int dir, const ExactOptions& opt,
                       double given_guess, int* converged) {
  Complete<D> sol = L;
  int iters = 0;
  int ok = 1;
  if (0.0 < L.rho && 0.0 < R.rho) {
    const StarState st = ComputeMiddleState<D>(eq, L, R, dir, opt.guess,
                                               given_guess, opt.tol,
                                               opt.max_iterations);
    iters = st.iterations;
    ok = st.converged;
    SampleRiemann<D>(eq, sol, L, R, dir, st.pM, st.uM);
  }
  Flux<D>(nf, sol, dir);
  if (converged) *converged = ok;
  return iters;
}

// Godunov::ComputeStableDt  include/fub/flux_method/GodunovMethod.hpp:173-183.
template <int D>
inline double GodunovStableDt(const Gas& eq, const Complete<D>& L,
                              const Complete<D>& R, double dx, int dir,
                              const ExactOptions& opt) {
  const StarState st = ComputeMiddleState<D>(eq, L, R, dir, opt.guess, 0.0,
                                             opt.tol, opt.max_iterations);
  double s0, s1;
  ExactSignals<D>(eq, L, R, dir, st.pM, s0, s1);
  double s_max = 0.0;
  s_max = std::max(s_max, std::abs(s0));
  s_max = std::max(s_max, std::abs(s1));
  return dx / s_max;
}

}  // namespace fvs_oracle
