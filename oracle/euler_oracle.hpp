// euler_oracle.hpp -- CPU oracle: point functions of the Euler equations,
// restated from PDESolver.jl (FP64, scalar-generic so that forward-mode dual
// numbers give exact derivatives).
//
// TEST INFRASTRUCTURE.  Only tests/, __graft_entry__.smoke() and bench.py's
// CPU-baseline leg may load this code.  It checks the GPU library; it is never
// the product path.
#pragma once
#include <cmath>
#include <algorithm>

namespace oracle {

// ---------------------------------------------------------------- dual numbers
// Forward-mode derivative carrier used for the oracle Jacobian (the reference
// derives its *_diff routines by hand; the same chain rule is applied here
// mechanically).
template <int N>
struct Dual {
  double v;
  double d[N];
  Dual() : v(0) { for (int i = 0; i < N; ++i) d[i] = 0; }
  Dual(double x) : v(x) { for (int i = 0; i < N; ++i) d[i] = 0; }  // NOLINT
};
template <int N> inline Dual<N> operator+(const Dual<N>& a, const Dual<N>& b) { Dual<N> r; r.v = a.v + b.v; for (int i = 0; i < N; ++i) r.d[i] = a.d[i] + b.d[i]; return r; }
template <int N> inline Dual<N> operator-(const Dual<N>& a, const Dual<N>& b) { Dual<N> r; r.v = a.v - b.v; for (int i = 0; i < N; ++i) r.d[i] = a.d[i] - b.d[i]; return r; }
template <int N> inline Dual<N> operator-(const Dual<N>& a) { Dual<N> r; r.v = -a.v; for (int i = 0; i < N; ++i) r.d[i] = -a.d[i]; return r; }
template <int N> inline Dual<N> operator*(const Dual<N>& a, const Dual<N>& b) { Dual<N> r; r.v = a.v * b.v; for (int i = 0; i < N; ++i) r.d[i] = a.d[i] * b.v + a.v * b.d[i]; return r; }
template <int N> inline Dual<N> operator/(const Dual<N>& a, const Dual<N>& b) { Dual<N> r; r.v = a.v / b.v; for (int i = 0; i < N; ++i) r.d[i] = (a.d[i] - r.v * b.d[i]) / b.v; return r; }
template <int N> inline Dual<N> operator+(const Dual<N>& a, double b) { Dual<N> r = a; r.v += b; return r; }
template <int N> inline Dual<N> operator+(double b, const Dual<N>& a) { return a + b; }
template <int N> inline Dual<N> operator-(const Dual<N>& a, double b) { Dual<N> r = a; r.v -= b; return r; }
template <int N> inline Dual<N> operator-(double b, const Dual<N>& a) { return Dual<N>(b) - a; }
template <int N> inline Dual<N> operator*(const Dual<N>& a, double b) { Dual<N> r; r.v = a.v * b; for (int i = 0; i < N; ++i) r.d[i] = a.d[i] * b; return r; }
template <int N> inline Dual<N> operator*(double b, const Dual<N>& a) { return a * b; }
template <int N> inline Dual<N> operator/(const Dual<N>& a, double b) { Dual<N> r; r.v = a.v / b; for (int i = 0; i < N; ++i) r.d[i] = a.d[i] / b; return r; }
template <int N> inline Dual<N> operator/(double a, const Dual<N>& b) { return Dual<N>(a) / b; }
template <int N> inline Dual<N>& operator+=(Dual<N>& a, const Dual<N>& b) { a = a + b; return a; }
template <int N> inline Dual<N>& operator-=(Dual<N>& a, const Dual<N>& b) { a = a - b; return a; }
template <int N> inline bool operator<(const Dual<N>& a, const Dual<N>& b) { return a.v < b.v; }
template <int N> inline bool operator<(const Dual<N>& a, double b) { return a.v < b; }
template <int N> inline Dual<N> sqrt(const Dual<N>& a) { Dual<N> r; r.v = std::sqrt(a.v); for (int i = 0; i < N; ++i) r.d[i] = a.d[i] / (2 * r.v); return r; }
template <int N> inline Dual<N> log(const Dual<N>& a) { Dual<N> r; r.v = std::log(a.v); for (int i = 0; i < N; ++i) r.d[i] = a.d[i] / a.v; return r; }
template <int N> inline Dual<N> absvalue(const Dual<N>& a) { return a.v < 0 ? -a : a; }
template <int N> inline Dual<N> maxval(const Dual<N>& a, const Dual<N>& b) { return (a.v >= b.v) ? a : b; }
template <int N> inline double real(const Dual<N>& a) { return a.v; }

inline double absvalue(double a) { return std::fabs(a); }
inline double maxval(double a, double b) { return std::max(a, b); }
inline double real(double a) { return a; }
using std::sqrt;
using std::log;

struct Params {
  double gamma, gamma_1;
  double Ma, aoa, rho_free, p_free, E_free;
  double r_in, rho_in, M_in;
  double R, cv;  // gas constant and cv = R/(gamma-1) (types.jl:242-244)
};

// ------------------------------------------------------------ calcPressure
// euler_funcs.jl:856-911
template <int DIM, typename T>
inline T pressure(const Params& p, const T* q) {
  if (DIM == 2) return p.gamma_1 * (q[3] - 0.5 * (q[1] * q[1] + q[2] * q[2]) / q[0]);
  return p.gamma_1 * (q[4] - 0.5 * (q[1] * q[1] + q[2] * q[2] + q[3] * q[3]) / q[0]);
}

// ------------------------------------------------------------ calcEulerFlux
// euler_funcs.jl:512-540 (2D), 749-773 (3D)
template <int DIM, typename T, typename Tn>
inline void euler_flux(const Params& p, const T* q, const Tn* dir, T* F) {
  T press = pressure<DIM>(p, q);
  if (DIM == 2) {
    T U = (q[1] * dir[0] + q[2] * dir[1]) / q[0];
    F[0] = q[0] * U;
    F[1] = q[1] * U + dir[0] * press;
    F[2] = q[2] * U + dir[1] * press;
    F[3] = (q[3] + press) * U;
  } else {
    T U = (q[1] * dir[0] + q[2] * dir[1] + q[3] * dir[2]) / q[0];
    F[0] = q[0] * U;
    F[1] = q[1] * U + dir[0] * press;
    F[2] = q[2] * U + dir[1] * press;
    F[3] = q[3] * U + dir[2] * press;
    F[4] = (q[4] + press) * U;
  }
}

// ------------------------------------------------------------ calcSAT
// bc_solvers.jl:207-311 (2D), 313-425 (3D): 0.5 (|A_hat| - A_hat)(qL - qR)
// with the eigenvalue floors sat_Vn = sat_Vl = 0.025.
template <int DIM, typename T, typename Tn>
inline void calc_sat(const Params& p, const T* roe, const T* dq, const Tn* nrm, T* sat) {
  const double sat_Vn = 0.025, sat_Vl = 0.025, tau = 1.0;
  const double gami = p.gamma_1;
  const int nv = DIM + 2;
  T u = roe[0], v = roe[1];
  T w = (DIM == 3) ? roe[2] : T(0.0);
  T H = roe[DIM];
  Tn nx = nrm[0], ny = nrm[1];
  Tn nz = (DIM == 3) ? nrm[2] : Tn(0.0);
  Tn dA = sqrt(nx * nx + ny * ny + nz * nz);
  T Un = u * nx + v * ny + w * nz;
  T phi = 0.5 * (u * u + v * v + w * w);
  T a = sqrt(gami * (H - phi));
  T lambda1 = Un + dA * a;
  T lambda2 = Un - dA * a;
  T lambda3 = Un;
  T rhoA = absvalue(Un) + dA * a;
  lambda1 = 0.5 * (tau * maxval(absvalue(lambda1), sat_Vn * rhoA) - lambda1);
  lambda2 = 0.5 * (tau * maxval(absvalue(lambda2), sat_Vn * rhoA) - lambda2);
  lambda3 = 0.5 * (tau * maxval(absvalue(lambda3), sat_Vl * rhoA) - lambda3);
  T E1dq[5], E2dq[5];
  for (int i = 0; i < nv; ++i) sat[i] = lambda3 * dq[i];
  // E1*dq
  T dqE = (DIM == 2) ? (phi * dq[0] - u * dq[1] - v * dq[2] + dq[3])
                     : (phi * dq[0] - u * dq[1] - v * dq[2] - w * dq[3] + dq[4]);
  T dqN = (DIM == 2) ? (-Un * dq[0] + nx * dq[1] + ny * dq[2])
                     : (-Un * dq[0] + nx * dq[1] + ny * dq[2] + nz * dq[3]);
  E1dq[0] = dqE; E1dq[1] = dqE * u; E1dq[2] = dqE * v;
  if (DIM == 3) E1dq[3] = dqE * w;
  E1dq[nv - 1] = dqE * H;
  // E2*dq
  E2dq[0] = T(0.0); E2dq[1] = dqN * nx; E2dq[2] = dqN * ny;
  if (DIM == 3) E2dq[3] = dqN * nz;
  E2dq[nv - 1] = dqN * Un;
  T tmp1 = 0.5 * (lambda1 + lambda2) - lambda3;
  T tmp2 = gami / (a * a);
  Tn tmp3 = 1.0 / (dA * dA);
  for (int i = 0; i < nv; ++i) sat[i] = sat[i] + tmp1 * (tmp2 * E1dq[i] + tmp3 * E2dq[i]);
  // E3*dq and E4*dq
  E1dq[0] = dqN; E1dq[1] = dqN * u; E1dq[2] = dqN * v;
  if (DIM == 3) E1dq[3] = dqN * w;
  E1dq[nv - 1] = dqN * H;
  E2dq[0] = T(0.0); E2dq[1] = dqE * nx; E2dq[2] = dqE * ny;
  if (DIM == 3) E2dq[3] = dqE * nz;
  E2dq[nv - 1] = dqE * Un;
  tmp1 = 0.5 * (lambda1 - lambda2) / (dA * a);
  for (int i = 0; i < nv; ++i) sat[i] = sat[i] + tmp1 * (E1dq[i] + gami * E2dq[i]);
}

// ------------------------------------------------------------ RoeSolver
// bc_solvers.jl:29-109 (2D), 111-205 (3D): F = F_euler(q).n + SAT
template <int DIM, typename T, typename Tn>
inline void roe_solver(const Params& p, const T* q, const T* qg, const Tn* nrm, T* flux) {
  const int nv = DIM + 2;
  const double gamma = p.gamma, gami = p.gamma_1;
  T fac = 1.0 / q[0];
  T uL = q[1] * fac, vL = q[2] * fac;
  T wL = (DIM == 3) ? q[3] * fac : T(0.0);
  T phi = 0.5 * (uL * uL + vL * vL + wL * wL);
  T HL = gamma * q[nv - 1] * fac - gami * phi;
  fac = 1.0 / qg[0];
  T uR = qg[1] * fac, vR = qg[2] * fac;
  T wR = (DIM == 3) ? qg[3] * fac : T(0.0);
  phi = 0.5 * (uR * uR + vR * vR + wR * wR);
  T HR = gamma * qg[nv - 1] * fac - gami * phi;
  T sqL = sqrt(q[0]);
  T sqR = sqrt(qg[0]);
  fac = 1.0 / (sqL + sqR);
  T roe[4];
  roe[0] = (sqL * uL + sqR * uR) * fac;
  roe[1] = (sqL * vL + sqR * vR) * fac;
  if (DIM == 3) roe[2] = (sqL * wL + sqR * wR) * fac;
  roe[DIM] = (sqL * HL + sqR * HR) * fac;
  T dq[5], sat[5], ef[5];
  for (int i = 0; i < nv; ++i) dq[i] = q[i] - qg[i];
  calc_sat<DIM>(p, roe, dq, nrm, sat);
  euler_flux<DIM>(p, q, nrm, ef);
  for (int i = 0; i < nv; ++i) flux[i] = sat[i] + ef[i];
}

// ------------------------------------------------------------ noPenetrationESBC
// bc.jl:767-795.  getDirichletState (bc.jl:860-919): qg = q with the normal
// momentum reversed, qg_m = -2 (n^ . m) n^ + m with n^ = nrm / |nrm|.
template <int DIM, typename T>
inline void nopenetration_state(const T* q, const double* nrm, T* qg) {
  double n2 = 0;
  for (int k = 0; k < DIM; ++k) n2 += nrm[k] * nrm[k];
  const double fac = 1.0 / std::sqrt(n2);
  double nh[3];
  for (int k = 0; k < DIM; ++k) nh[k] = nrm[k] * fac;
  T Unrm = T(0.0);
  for (int k = 0; k < DIM; ++k) Unrm = Unrm + nh[k] * q[1 + k];
  qg[0] = q[0];
  for (int k = 0; k < DIM; ++k) qg[1 + k] = -2 * Unrm * nh[k] + q[1 + k];
  qg[DIM + 1] = q[DIM + 1];
}

// getLambdaMax (euler_funcs.jl:1887-1910): |U . dir| + |dir| a
template <int DIM, typename T>
inline T lambda_max(const Params& p, const T* q, const double* dir) {
  T rhoinv = 1.0 / q[0];
  T pr = pressure<DIM>(p, q);
  T a = sqrt(p.gamma * pr * rhoinv);
  T Un = T(0.0);
  double dA = 0;
  for (int i = 0; i < DIM; ++i) {
    Un = Un + dir[i] * q[i + 1] * rhoinv;
    dA += dir[i] * dir[i];
  }
  return absvalue(Un) + std::sqrt(dA) * a;
}

// calcLFFlux (bc_solvers.jl:428-446) with getLambdaMaxSimple
// (IR_stab.jl:310-326: lambda_max at the arithmetic mean of the states)
template <int DIM, typename T>
inline void lf_flux(const Params& p, const T* qL, const T* qR, const double* dir, T* F) {
  const int nv = DIM + 2;
  T fL[5], fR[5], qa[5];
  euler_flux<DIM>(p, qL, dir, fL);
  euler_flux<DIM>(p, qR, dir, fR);
  for (int i = 0; i < nv; ++i) qa[i] = 0.5 * (qL[i] + qR[i]);
  T lam = lambda_max<DIM>(p, qa, dir);
  for (int i = 0; i < nv; ++i) F[i] = 0.5 * (fL[i] + fR[i] - lam * (qR[i] - qL[i]));
}

// the boundary flux of noPenetrationESBC at one face node
template <int DIM, typename T>
inline void nopenetration_es_flux(const Params& p, const T* q, const double* nrm, T* F) {
  T qg[5];
  nopenetration_state<DIM>(q, nrm, qg);
  lf_flux<DIM>(p, q, qg, nrm, F);
}

// ------------------------------------------------------------ logavg
// bc_solvers.jl:942-956: logarithmic mean, 5-term series for u < 1e-3
template <typename T>
inline T logavg(const T& aL, const T& aR) {
  T xi = aL / aR;
  T f = (xi - 1.0) / (xi + 1.0);
  T u = f * f;
  T F;
  if (real(u) < 1e-3) {
    F = 1.0 + u * (1.0 / 3.0 + u * (1.0 / 5.0 + u * (1.0 / 7.0 + u * (1.0 / 9.0))));
  } else {
    F = (log(xi) / 2.0) / f;
  }
  return (aL + aR) / (2.0 * F);
}

// ------------------------------------------------------------ calcEulerFlux_IR
// bc_solvers.jl:725-884: Ismail-Roe entropy-conservative flux in ndir
// directions (dir[d][k]: component k of direction d).
template <int DIM, typename T, typename Tn>
inline void ir_flux(const Params& p, const T* qL, const T* qR, const Tn* dir, int ndir, T* F) {
  const int nv = DIM + 2;
  const double gamma = p.gamma, gamma_1 = p.gamma_1;
  T pL = pressure<DIM>(p, qL), pR = pressure<DIM>(p, qR);
  T z1L = sqrt(qL[0] / pL), z1R = sqrt(qR[0] / pR);
  T z2L = z1L * qL[1] / qL[0], z2R = z1R * qR[1] / qR[0];
  T z3L = z1L * qL[2] / qL[0], z3R = z1R * qR[2] / qR[0];
  T z4L = (DIM == 3) ? z1L * qL[3] / qL[0] : T(0.0);
  T z4R = (DIM == 3) ? z1R * qR[3] / qR[0] : T(0.0);
  T zpL = sqrt(qL[0] * pL), zpR = sqrt(qR[0] * pR);
  T lp = logavg(zpL, zpR);
  T rho_hat = 0.5 * (z1L + z1R) * lp;
  T u_hat = (z2L + z2R) / (z1L + z1R);
  T v_hat = (z3L + z3R) / (z1L + z1R);
  T w_hat = (z4L + z4R) / (z1L + z1R);
  T p1_hat = (zpL + zpR) / (z1L + z1R);
  T p2_hat = ((gamma + 1) / (2 * gamma)) * lp / logavg(z1L, z1R) +
             (gamma_1 / (2 * gamma)) * (zpL + zpR) / (z1L + z1R);
  T h_hat = gamma * p2_hat / (rho_hat * gamma_1) + 0.5 * (u_hat * u_hat + v_hat * v_hat + w_hat * w_hat);
  for (int d = 0; d < ndir; ++d) {
    const Tn* n = dir + d * DIM;
    Tn nz = (DIM == 3) ? n[2] : Tn(0.0);
    T mv_n = rho_hat * (n[0] * u_hat + n[1] * v_hat + nz * w_hat);
    T* Fd = F + d * nv;
    Fd[0] = mv_n;
    Fd[1] = mv_n * u_hat + n[0] * p1_hat;
    Fd[2] = mv_n * v_hat + n[1] * p1_hat;
    if (DIM == 3) Fd[3] = mv_n * w_hat + nz * p1_hat;
    Fd[nv - 1] = mv_n * h_hat;
  }
}

// ------------------------------------------------------------ states
// calcIsentropicVortex, common_funcs.jl:25-79 (with M_in a parameter)
inline void isentropic_vortex(const Params& p, const double* x, double* sol) {
  double gamma = p.gamma;
  double r_in = p.r_in, rho_in = p.rho_in, M_in = p.M_in, p_in = 1.0 / gamma;
  double r = std::sqrt(x[0] * x[0] + x[1] * x[1]);
  double theta = std::atan2(x[1], x[0]);
  double tmp1 = ((gamma - 1) / 2) * M_in * M_in;
  double rho_r = rho_in * std::pow(1 + tmp1 * (1 - (r_in * r_in) / (r * r)), 1 / (gamma - 1));
  double p_r = p_in * std::pow(rho_r / rho_in, gamma);
  double a_r = std::sqrt(gamma * p_r / rho_r);
  double M_r = std::sqrt((2 / (gamma - 1)) * std::pow(rho_in / rho_r, gamma - 1) * (1 + tmp1) - 2 / (gamma - 1));
  double U_r = M_r * a_r;
  double u_r = U_r * std::sin(theta);
  double v_r = -U_r * std::cos(theta);
  double e_r = p.cv * p_r / (rho_r * p.R);
  double E_r = rho_r * e_r + 0.5 * rho_r * U_r * U_r;
  sol[0] = rho_r;
  sol[1] = rho_r * u_r;
  sol[2] = rho_r * v_r;
  sol[3] = E_r;
}

// calcFreeStream, common_funcs.jl:312-345
template <int DIM>
inline void free_stream(const Params& p, double* sol) {
  double rho = p.rho_free;
  sol[0] = rho;
  sol[DIM + 1] = p.E_free;
  sol[1] = rho * p.Ma * std::cos(p.aoa);
  if (DIM == 2) {
    sol[2] = rho * p.Ma * std::sin(p.aoa);
  } else {
    sol[2] = 0.0;
    sol[3] = -rho * p.Ma * std::sin(p.aoa);
  }
}

}  // namespace oracle
