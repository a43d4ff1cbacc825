// eg_physics.cuh -- point functions of the Euler equations on the device.
//
// Scalar-generic (T = double, float, or a forward-mode derivative carrier) so
// the Jacobian kernels differentiate the same arithmetic the residual uses.
// Formulas follow the reference:
//   calcPressure      src/solver/euler/euler_funcs.jl:856-911
//   calcEulerFlux     src/solver/euler/euler_funcs.jl:512-540, 749-773
//   RoeSolver/calcSAT src/solver/euler/bc_solvers.jl:29-425
//   calcEulerFlux_IR  src/solver/euler/bc_solvers.jl:725-884
//   logavg            src/solver/euler/bc_solvers.jl:942-956
#pragma once
#include <cuda_runtime.h>

#include <type_traits>

namespace eg {

// ---------------------------------------------------------------------------
// derivative carrier: value + N directional derivatives
template <typename R, int N>
struct Fwd {
  R v;
  R d[N];
  __host__ __device__ Fwd() {}
  __host__ __device__ Fwd(R x) : v(x) {  // NOLINT: implicit from constants
#pragma unroll
    for (int i = 0; i < N; ++i) d[i] = R(0);
  }
};

#define EG_FWD_BIN(OP, VAL, DER)                                                             \
  template <typename R, int N>                                                               \
  __host__ __device__ __forceinline__ Fwd<R, N> operator OP(const Fwd<R, N>& a,              \
                                                            const Fwd<R, N>& b) {            \
    Fwd<R, N> r;                                                                             \
    r.v = VAL;                                                                               \
    _Pragma("unroll") for (int i = 0; i < N; ++i) r.d[i] = DER;                              \
    return r;                                                                                \
  }
EG_FWD_BIN(+, a.v + b.v, a.d[i] + b.d[i])
EG_FWD_BIN(-, a.v - b.v, a.d[i] - b.d[i])
EG_FWD_BIN(*, a.v * b.v, a.d[i] * b.v + a.v * b.d[i])
#undef EG_FWD_BIN

template <typename R, int N>
__host__ __device__ __forceinline__ Fwd<R, N> operator/(const Fwd<R, N>& a, const Fwd<R, N>& b) {
  Fwd<R, N> r;
  R ib = R(1) / b.v;
  r.v = a.v * ib;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = (a.d[i] - r.v * b.d[i]) * ib;
  return r;
}
template <typename R, int N>
__host__ __device__ __forceinline__ Fwd<R, N> operator-(const Fwd<R, N>& a) {
  Fwd<R, N> r;
  r.v = -a.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = -a.d[i];
  return r;
}
// mixed with plain scalars (any arithmetic type, converted to R so an FP32
// carrier never issues FP64 instructions)
template <typename S>
struct IsScalar { static constexpr bool value = false; };
template <> struct IsScalar<double> { static constexpr bool value = true; };
template <> struct IsScalar<float> { static constexpr bool value = true; };
template <> struct IsScalar<int> { static constexpr bool value = true; };
#define EG_SCALAR_OK(S) typename = typename std::enable_if<IsScalar<S>::value>::type

template <typename R, int N, typename S, EG_SCALAR_OK(S)>
__host__ __device__ __forceinline__ Fwd<R, N> operator*(const Fwd<R, N>& a, S bs) {
  const R b = R(bs);
  Fwd<R, N> r;
  r.v = a.v * b;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] * b;
  return r;
}
template <typename R, int N, typename S, EG_SCALAR_OK(S)>
__host__ __device__ __forceinline__ Fwd<R, N> operator*(S b, const Fwd<R, N>& a) { return a * b; }
template <typename R, int N, typename S, EG_SCALAR_OK(S)>
__host__ __device__ __forceinline__ Fwd<R, N> operator+(const Fwd<R, N>& a, S b) { Fwd<R, N> r = a; r.v = a.v + R(b); return r; }
template <typename R, int N, typename S, EG_SCALAR_OK(S)>
__host__ __device__ __forceinline__ Fwd<R, N> operator+(S b, const Fwd<R, N>& a) { Fwd<R, N> r = a; r.v = R(b) + a.v; return r; }
template <typename R, int N, typename S, EG_SCALAR_OK(S)>
__host__ __device__ __forceinline__ Fwd<R, N> operator-(const Fwd<R, N>& a, S b) { Fwd<R, N> r = a; r.v = a.v - R(b); return r; }
template <typename R, int N, typename S, EG_SCALAR_OK(S)>
__host__ __device__ __forceinline__ Fwd<R, N> operator-(S b, const Fwd<R, N>& a) { return Fwd<R, N>(R(b)) - a; }
template <typename R, int N, typename S, EG_SCALAR_OK(S)>
__host__ __device__ __forceinline__ Fwd<R, N> operator/(const Fwd<R, N>& a, S b) { return a * (R(1) / R(b)); }
template <typename R, int N, typename S, EG_SCALAR_OK(S)>
__host__ __device__ __forceinline__ Fwd<R, N> operator/(S a, const Fwd<R, N>& b) { return Fwd<R, N>(R(a)) / b; }

template <typename R, int N>
__host__ __device__ __forceinline__ Fwd<R, N> sqrt(const Fwd<R, N>& a) {
  Fwd<R, N> r;
  r.v = ::sqrt(a.v);
  R h = R(0.5) / r.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] * h;
  return r;
}
template <typename R, int N>
__host__ __device__ __forceinline__ Fwd<R, N> log(const Fwd<R, N>& a) {
  Fwd<R, N> r;
  r.v = ::log(a.v);
  R ia = R(1) / a.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] * ia;
  return r;
}
template <typename R, int N>
__host__ __device__ __forceinline__ Fwd<R, N> absval(const Fwd<R, N>& a) { return a.v < R(0) ? -a : a; }
template <typename R, int N>
__host__ __device__ __forceinline__ Fwd<R, N> maxval(const Fwd<R, N>& a, const Fwd<R, N>& b) { return (a.v >= b.v) ? a : b; }
template <typename R, int N>
__host__ __device__ __forceinline__ R val(const Fwd<R, N>& a) { return a.v; }

__host__ __device__ __forceinline__ double absval(double a) { return fabs(a); }
__host__ __device__ __forceinline__ float absval(float a) { return fabsf(a); }
__host__ __device__ __forceinline__ double maxval(double a, double b) { return fmax(a, b); }
__host__ __device__ __forceinline__ float maxval(float a, float b) { return fmaxf(a, b); }
__host__ __device__ __forceinline__ double val(double a) { return a; }
__host__ __device__ __forceinline__ float val(float a) { return a; }
using ::sqrt;
using ::log;

// 1/sqrt(x): CUDA's rsqrt (double) / rsqrtf (float); for a derivative
// carrier d(x^-1/2) = -x^-3/2 dx / 2
__device__ __forceinline__ double rsqrt_(double a) { return ::rsqrt(a); }
__device__ __forceinline__ float rsqrt_(float a) { return ::rsqrtf(a); }
template <typename R, int N>
__device__ __forceinline__ Fwd<R, N> rsqrt_(const Fwd<R, N>& a) {
  Fwd<R, N> r;
  r.v = rsqrt_(a.v);
  const R dr = R(-0.5) * r.v * r.v * r.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] * dr;
  return r;
}

// real (non-derivative) type of a scalar
template <typename T> struct RealOf { using type = T; };
template <typename R, int N> struct RealOf<Fwd<R, N>> { using type = R; };

// gas constants as seen by the kernels
struct Gas {
  double gamma, gamma_1;
};

// ---------------------------------------------------------------------------
// Every literal below is converted to R = RealOf<T>, so an FP32 instantiation
// is FP32 throughout and the FP64 one is FP64 throughout.
template <int DIM, typename T>
__device__ __forceinline__ T pressure(const Gas& g, const T* q) {
  using R = typename RealOf<T>::type;
  const R h = R(0.5), g1 = R(g.gamma_1);
  if (DIM == 2) return g1 * (q[3] - h * (q[1] * q[1] + q[2] * q[2]) / q[0]);
  return g1 * (q[4] - h * (q[1] * q[1] + q[2] * q[2] + q[3] * q[3]) / q[0]);
}

// F . dir for the Euler equations (conservative variables)
template <int DIM, typename T, typename Tn>
__device__ __forceinline__ void euler_flux(const Gas& g, const T* q, const Tn* dir, T* F) {
  using R = typename RealOf<T>::type;
  const R h = R(0.5), g1 = R(g.gamma_1);
  const T r = R(1) / q[0];
  if (DIM == 2) {
    T press = g1 * (q[3] - h * (q[1] * q[1] + q[2] * q[2]) * r);
    T U = (q[1] * dir[0] + q[2] * dir[1]) * r;
    F[0] = q[0] * U;
    F[1] = q[1] * U + dir[0] * press;
    F[2] = q[2] * U + dir[1] * press;
    F[3] = (q[3] + press) * U;
  } else {
    T press = g1 * (q[4] - h * (q[1] * q[1] + q[2] * q[2] + q[3] * q[3]) * r);
    T U = (q[1] * dir[0] + q[2] * dir[1] + q[3] * dir[2]) * r;
    F[0] = q[0] * U;
    F[1] = q[1] * U + dir[0] * press;
    F[2] = q[2] * U + dir[1] * press;
    F[3] = q[3] * U + dir[2] * press;
    F[4] = (q[4] + press) * U;
  }
}

// Roe flux: F(qL).n + 0.5 (|A_hat| - A_hat)(qL - qR), eigenvalue floors 0.025.
// Arranged to spend one division (FP64 is the scarce resource on GB300):
// 1/(sqL + sqR).  Four reciprocal square roots give the rest:
//   s = rho^-1/2 of each state: sqrt(rho) = rho s and 1/rho = s^2;
//   rn = |n|^-1: |n| = n.n rn and 1/|n|^2 = rn^2;
//   ia = 1/a with a^2 = gami (H - phi): a = a^2 ia, 1/(H - phi) = gami ia^2
//   and 1/(|n| a) = rn ia.
// The Euler flux of qL reuses 1/rho_L.
template <int DIM, typename T, typename Tn>
__device__ __forceinline__ void roe_flux(const Gas& g, const T* q, const T* qg, const Tn* nrm, T* flux) {
  using R = typename RealOf<T>::type;
  constexpr int NV = DIM + 2;
  const R gamma = R(g.gamma), gami = R(g.gamma_1), h = R(0.5), one = R(1);
  const R sat_V = R(0.025);
  // Roe averages
  const T isL = rsqrt_(q[0]);
  const T rL = isL * isL;
  T uL = q[1] * rL, vL = q[2] * rL;
  T wL = (DIM == 3) ? q[3] * rL : T(R(0));
  T phiL = h * (uL * uL + vL * vL + wL * wL);
  T HL = gamma * q[NV - 1] * rL - gami * phiL;
  const T isR = rsqrt_(qg[0]);
  const T rR = isR * isR;
  T uR = qg[1] * rR, vR = qg[2] * rR;
  T wR = (DIM == 3) ? qg[3] * rR : T(R(0));
  T phiR = h * (uR * uR + vR * vR + wR * wR);
  T HR = gamma * qg[NV - 1] * rR - gami * phiR;
  T sqL = q[0] * isL;
  T sqR = qg[0] * isR;
  T fac = one / (sqL + sqR);
  T u = (sqL * uL + sqR * uR) * fac;
  T v = (sqL * vL + sqR * vR) * fac;
  T w = (DIM == 3) ? (sqL * wL + sqR * wR) * fac : T(R(0));
  T H = (sqL * HL + sqR * HR) * fac;
  T dq[NV];
#pragma unroll
  for (int i = 0; i < NV; ++i) dq[i] = q[i] - qg[i];
  // SAT
  Tn nx = nrm[0], ny = nrm[1];
  Tn nz = (DIM == 3) ? nrm[2] : Tn(0);
  Tn n2 = nx * nx + ny * ny + nz * nz;
  Tn rn = rsqrt_(n2);
  Tn dA = n2 * rn;
  T Un = u * nx + v * ny + w * nz;
  T phi = h * (u * u + v * v + w * w);
  T Hp = H - phi;
  T a2 = gami * Hp;
  T ia = rsqrt_(a2);
  T a = a2 * ia;
  T dAa = dA * a;
  T lambda1 = Un + dAa;
  T lambda2 = Un - dAa;
  T lambda3 = Un;
  T rhoA = absval(Un) + dAa;
  lambda1 = h * (maxval(absval(lambda1), sat_V * rhoA) - lambda1);
  lambda2 = h * (maxval(absval(lambda2), sat_V * rhoA) - lambda2);
  lambda3 = h * (maxval(absval(lambda3), sat_V * rhoA) - lambda3);
  T dqE, dqN;
  if (DIM == 2) {
    dqE = phi * dq[0] - u * dq[1] - v * dq[2] + dq[3];
    dqN = -Un * dq[0] + nx * dq[1] + ny * dq[2];
  } else {
    dqE = phi * dq[0] - u * dq[1] - v * dq[2] - w * dq[3] + dq[4];
    dqN = -Un * dq[0] + nx * dq[1] + ny * dq[2] + nz * dq[3];
  }
  T t1 = h * (lambda1 + lambda2) - lambda3;
  T t2 = gami * ia * ia;           // 1 / (H - phi) = gami / a^2
  Tn t3 = rn * rn;                 // 1 / dA^2
  T t4 = h * (lambda1 - lambda2) * (rn * ia);  // / (dA a)
  // sat = l3 dq + t1 (t2 E1dq + t3 E2dq) + t4 (E3dq + gami E4dq)
  T c1 = t1 * t2 * dqE + t4 * dqN;        // coefficient of (1, u, v, w, H)
  T c2 = t1 * t3 * dqN + t4 * gami * dqE; // coefficient of (0, nx, ny, nz, Un)
  // Euler flux of qL in direction n, reusing 1/rho_L
  T ke = q[1] * q[1] + q[2] * q[2];
  if (DIM == 3) ke = ke + q[3] * q[3];
  T pL = gami * (q[NV - 1] - h * ke * rL);
  T UL = q[1] * nx + q[2] * ny;
  if (DIM == 3) UL = UL + q[3] * nz;
  UL = UL * rL;
  flux[0] = q[0] * UL + lambda3 * dq[0] + c1;
  flux[1] = q[1] * UL + nx * pL + lambda3 * dq[1] + c1 * u + c2 * nx;
  flux[2] = q[2] * UL + ny * pL + lambda3 * dq[2] + c1 * v + c2 * ny;
  if (DIM == 3) flux[3] = q[3] * UL + nz * pL + lambda3 * dq[3] + c1 * w + c2 * nz;
  flux[NV - 1] = (q[NV - 1] + pL) * UL + lambda3 * dq[NV - 1] + c1 * H + c2 * Un;
}

// Entropy-stable no-penetration wall (reference noPenetrationESBC,
// bc.jl:767-795): the mirror state qg = q with the normal momentum reversed,
// m_g = m - 2 (m . n^) n^ (getDirichletState, bc.jl:860-919), and the
// Lax-Friedrichs flux between q and qg (calcLFFlux, bc_solvers.jl:428-446):
// F = (F(q).n + F(qg).n - lambda_max (qg - q)) / 2, lambda_max = |U_n| +
// |n| a at the mean state (q + qg) / 2 (getLambdaMaxSimple, IR_stab.jl:
// 310-326; getLambdaMax, euler_funcs.jl:1887-1910).  Scalar-generic: with a
// derivative carrier q the derivative runs through qg as well.
template <int DIM, typename T, typename Tn>
__device__ __forceinline__ void wall_es_flux(const Gas& g, const T* q, const Tn* nrm, T* flux) {
  using R = typename RealOf<T>::type;
  constexpr int NV = DIM + 2;
  const R h = R(0.5), two = R(2), gamma = R(g.gamma);
  Tn n2 = nrm[0] * nrm[0] + nrm[1] * nrm[1];
  if (DIM == 3) n2 = n2 + nrm[2] * nrm[2];
  const Tn dA = sqrt(n2);
  const Tn fac = Tn(1) / dA;
  Tn nh[DIM];
#pragma unroll
  for (int k = 0; k < DIM; ++k) nh[k] = nrm[k] * fac;
  T Unrm = q[1] * nh[0] + q[2] * nh[1];
  if (DIM == 3) Unrm = Unrm + q[3] * nh[2];
  T qg[NV];
  qg[0] = q[0];
#pragma unroll
  for (int k = 0; k < DIM; ++k) qg[1 + k] = q[1 + k] - two * Unrm * nh[k];
  qg[NV - 1] = q[NV - 1];
  T FL[NV], FR[NV];
  euler_flux<DIM>(g, q, nrm, FL);
  euler_flux<DIM>(g, qg, nrm, FR);
  T qa[NV];
#pragma unroll
  for (int c = 0; c < NV; ++c) qa[c] = h * (q[c] + qg[c]);
  const T ra = R(1) / qa[0];
  const T pa = pressure<DIM>(g, qa);
  const T aa = sqrt(gamma * pa * ra);
  T Un = nrm[0] * qa[1] * ra + nrm[1] * qa[2] * ra;
  if (DIM == 3) Un = Un + nrm[2] * qa[3] * ra;
  const T lam = absval(Un) + dA * aa;
#pragma unroll
  for (int c = 0; c < NV; ++c) flux[c] = h * (FL[c] + FR[c] - lam * (qg[c] - q[c]));
}

// logarithmic mean with the 5-term series below u = 1e-3
template <typename T>
__device__ __forceinline__ T logavg(const T& aL, const T& aR) {
  using R = typename RealOf<T>::type;
  const R one = R(1);
  T xi = aL / aR;
  T f = (xi - one) / (xi + one);
  T u = f * f;
  T F;
  if (val(u) < R(1e-3)) {
    F = one + u * (R(1.0 / 3.0) + u * (R(1.0 / 5.0) + u * (R(1.0 / 7.0) + u * R(1.0 / 9.0))));
  } else {
    F = (log(xi) * R(0.5)) / f;
  }
  return (aL + aR) / (R(2) * F);
}

// Ismail-Roe flux: shared averages, then NDIR directions dir[d*DIM + k]
template <int DIM, typename T>
struct IRAvg {
  T rho_hat, u_hat, v_hat, w_hat, p1_hat, h_hat;
};

template <int DIM, typename T>
__device__ __forceinline__ IRAvg<DIM, T> ir_average(const Gas& g, const T* qL, const T* qR) {
  using R = typename RealOf<T>::type;
  const R gamma = R(g.gamma), gamma_1 = R(g.gamma_1), h = R(0.5), one = R(1);
  T pL = pressure<DIM>(g, qL), pR = pressure<DIM>(g, qR);
  T z1L = sqrt(qL[0] / pL), z1R = sqrt(qR[0] / pR);
  T zpL = sqrt(qL[0] * pL), zpR = sqrt(qR[0] * pR);
  T iz = one / (z1L + z1R);
  IRAvg<DIM, T> r;
  T lp = logavg(zpL, zpR);
  r.rho_hat = h * (z1L + z1R) * lp;
  r.u_hat = (z1L * qL[1] / qL[0] + z1R * qR[1] / qR[0]) * iz;
  r.v_hat = (z1L * qL[2] / qL[0] + z1R * qR[2] / qR[0]) * iz;
  r.w_hat = (DIM == 3) ? (z1L * qL[3] / qL[0] + z1R * qR[3] / qR[0]) * iz : T(R(0));
  r.p1_hat = (zpL + zpR) * iz;
  T p2_hat = R((g.gamma + 1) / (2 * g.gamma)) * lp / logavg(z1L, z1R) +
             R(g.gamma_1 / (2 * g.gamma)) * (zpL + zpR) * iz;
  r.h_hat = gamma * p2_hat / (r.rho_hat * gamma_1) +
            h * (r.u_hat * r.u_hat + r.v_hat * r.v_hat + r.w_hat * r.w_hat);
  return r;
}

// Per-node quantities of the Ismail-Roe averages: z1 = sqrt(rho/p),
// zp = sqrt(rho p), their logarithms and the velocity.  Computed once per node
// so a pair of nodes needs no square root and no logarithm.
template <int DIM>
struct IRNode {
  double z1, zp, lz1, lzp, u, v, w;
};

template <int DIM, bool LOGS = true>
__device__ __forceinline__ IRNode<DIM> ir_node(const Gas& g, const double* q) {
  IRNode<DIM> r;
  const double p = pressure<DIM>(g, q);
  // t = (rho p)^-1/2: sqrt(rho/p) = rho t, sqrt(rho p) = rho p t, 1/rho = p t^2
  const double t = rsqrt_(q[0] * p);
  const double rinv = p * t * t;
  r.z1 = q[0] * t;
  r.zp = q[0] * p * t;
  if (LOGS) {
    r.lz1 = log(r.z1);
    r.lzp = log(r.zp);
  } else {
    r.lz1 = r.lzp = 0.0;
  }
  r.u = q[1] * rinv;
  r.v = q[2] * rinv;
  r.w = (DIM == 3) ? q[3] * rinv : 0.0;
  return r;
}

// Logarithmic means for the Ismail-Roe average from precomputed logarithms.
// The reference's logavg (bc_solvers.jl:942-956) is (aL + aR) / (2 F) with
// u = f^2, f = (aL - aR)/(aL + aR), and F = 1 + u/3 + u^2/5 + u^3/7 + u^4/9
// for u < 1e-3, else F = ln(aL/aR) / (2 f).  The average needs the log mean of
// sqrt(rho p) (L_p), its reciprocal, and the reciprocal of the log mean of
// sqrt(rho/p) (1/L_1); all three follow from 1/(aL + aR) and F:
//   L = s/(2F) = (s/2) G(u),  1/L = 2 F / s,
// with G = 1/F as its series 1 - u/3 - 4u^2/45 - 44u^3/945 - 428u^4/14175
// (|G F - 1| < 5e-16 for u < 1e-3), and in the logarithmic branch
//   1/L = (lL - lR)/d,  L = d^2 x and 1/L = (lL - lR)^2 x with x = 1/(d (lL - lR)).
// A pair costs one division on the series branch: x = 1/(s_1 s_p) gives
// 1/s_1 = s_p x and 1/s_p = s_1 x.
__device__ __forceinline__ double logmean_F(double u) {
  return 1.0 + u * (1.0 / 3.0 + u * (1.0 / 5.0 + u * (1.0 / 7.0 + u * (1.0 / 9.0))));
}
__device__ __forceinline__ double logmean_G(double u) {
  return 1.0 - u * (1.0 / 3.0 + u * (4.0 / 45.0 + u * (44.0 / 945.0 + u * (428.0 / 14175.0))));
}

// Ismail-Roe averages of two nodes from their per-node quantities.  PRE: the
// nodes carry their logarithms (computed once per node, for the pairs of an
// element); otherwise the logarithm of the ratio is taken on the log-mean
// branch only (a face node pairs each state once).
template <int DIM, bool PRE = true>
__device__ __forceinline__ IRAvg<DIM, double> ir_average_pre(const Gas& g, const IRNode<DIM>& L,
                                                             const IRNode<DIM>& R) {
  const double gamma = g.gamma, gamma_1 = g.gamma_1;
  IRAvg<DIM, double> r;
  // sqrt(rho/p): r1 = 1/(z1L + z1R) is also the weight of the velocity averages;
  // one division for 1/s1 and 1/sp
  const double s1 = L.z1 + R.z1, d1 = L.z1 - R.z1;
  const double sp = L.zp + R.zp, dp = L.zp - R.zp;
  const double x1p = 1.0 / (s1 * sp);
  const double r1 = sp * x1p;
  double inv_l1;
  if (d1 * d1 < 1e-3 * (s1 * s1)) {
    const double f = d1 * r1;
    inv_l1 = 2.0 * logmean_F(f * f) * r1;
  } else {
    inv_l1 = (PRE ? L.lz1 - R.lz1 : log(L.z1 / R.z1)) / d1;
  }
  // sqrt(rho p)
  double lp, inv_lp;
  if (dp * dp < 1e-3 * (sp * sp)) {
    const double rp = s1 * x1p;
    const double f = dp * rp, u = f * f;
    lp = 0.5 * sp * logmean_G(u);
    inv_lp = 2.0 * logmean_F(u) * rp;
  } else {
    const double dl = PRE ? L.lzp - R.lzp : log(L.zp / R.zp);
    const double x = 1.0 / (dp * dl);
    lp = dp * dp * x;
    inv_lp = dl * dl * x;
  }
  r.rho_hat = 0.5 * s1 * lp;
  r.u_hat = (L.z1 * L.u + R.z1 * R.u) * r1;
  r.v_hat = (L.z1 * L.v + R.z1 * R.v) * r1;
  r.w_hat = (DIM == 3) ? (L.z1 * L.w + R.z1 * R.w) * r1 : 0.0;
  r.p1_hat = sp * r1;
  const double p2_hat = ((gamma + 1) / (2 * gamma)) * lp * inv_l1 + (gamma_1 / (2 * gamma)) * r.p1_hat;
  // h = gamma p2 / (rho_hat (gamma - 1)) + |u|^2/2, 1/rho_hat = 2 r1 / L_p
  r.h_hat = (gamma / gamma_1) * p2_hat * (2.0 * r1 * inv_lp) +
            0.5 * (r.u_hat * r.u_hat + r.v_hat * r.v_hat + r.w_hat * r.w_hat);
  return r;
}

template <int DIM, typename T, typename Tn>
__device__ __forceinline__ void ir_dir(const IRAvg<DIM, T>& a, const Tn* n, T* F) {
  constexpr int NV = DIM + 2;
  Tn nz = (DIM == 3) ? n[2] : Tn(0);
  T mv_n = a.rho_hat * (n[0] * a.u_hat + n[1] * a.v_hat + nz * a.w_hat);
  F[0] = mv_n;
  F[1] = mv_n * a.u_hat + n[0] * a.p1_hat;
  F[2] = mv_n * a.v_hat + n[1] * a.p1_hat;
  if (DIM == 3) F[3] = mv_n * a.w_hat + nz * a.p1_hat;
  F[NV - 1] = mv_n * a.h_hat;
}

}  // namespace eg
