// Second-order (MUSCL) residual with SSP-RK3 / forward-Euler stages.
//
// No reference counterpart: the reference is first-order in space and time
// (docs/dns-higher-order-scheme-plan.md:52-95 sketches this form).  The CPU
// FP64 definition these kernels are checked against is
// oracle/fv_oracle.cpp (Euler::gradients / recon / residual / step).
//
// Per RK stage, three passes over HBM-resident arrays:
//   k_grad   one thread per cell: gradients of the primitive variables
//            (rho, u, v, p) by weighted least squares (weights pre-folded
//            with the inverse normal matrix, one pair per CSR entry) or
//            Green-Gauss, then Barth-Jespersen or Venkatakrishnan limiting.
//            The per-face limiter values are min-reduced by
//            cross-multiplication, so each variable costs one reciprocal.
//   k_face   one thread per face: linear reconstruction to the face
//            midpoint (positivity fallback to the cell value), ghost state
//            from the reconstructed owner state, numerical flux on
//            primitive inputs; at stage 0 also the face's CFL time step.
//   k_update one thread per cell: FP64 signed gather of the face fluxes in
//            the reference's per-cell face order, stage-0 time step and
//            residual norms, the Shu-Osher stage combination, and the
//            primitive copy W (flux precision) + sound speed for the next
//            stage.
//
// T is the flux/gradient arithmetic type: double (FP64 mode) or float
// (FP32-flux mode).  Residual accumulation, the state update, dt and the
// norms are always FP64.
#pragma once

#include <type_traits>

#include "euler_o1.cuh"
#include "fpconv.cuh"

namespace FV_KNS {

template <typename T> struct V4 { T r, u, v, p; };
template <typename T> struct G8 { T gx[4], gy[4]; };

template <typename T> __device__ __forceinline__ T tsqrt(T x);
template <> __device__ __forceinline__ double tsqrt<double>(double x) { return sqrt(x); }
template <> __device__ __forceinline__ float tsqrt<float>(float x) { return sqrtf(x); }
template <typename T> __device__ __forceinline__ T tpow(T a, T b);
template <> __device__ __forceinline__ double tpow<double>(double a, double b) { return pow(a, b); }
template <> __device__ __forceinline__ float tpow<float>(float a, float b) { return powf(a, b); }

// W storage: double -> 32-byte {r,u,v,p}; float -> float4.
template <typename T> struct WStore;
template <> struct WStore<double> {
    using type = St;
    __device__ static V4<double> ld(const St* W, int i) {
        St s = ld_state(W, i);
        return {s.r, s.ru, s.rv, s.E};
    }
    __device__ static void st(St* W, int i, const V4<double>& w) { st_state(W, i, st_make(w.r, w.u, w.v, w.p)); }
};
template <> struct WStore<float> {
    using type = float4;
    __device__ static V4<float> ld(const float4* W, int i) {
        float4 a = __ldg(W + i);
        return {a.x, a.y, a.z, a.w};
    }
    __device__ static void st(float4* W, int i, const V4<float>& w) { W[i] = make_float4(w.r, w.u, w.v, w.p); }
};

template <typename T> struct GStore;
template <> struct GStore<double> {
    using type = double2;  // 4 x double2 per cell: (gx,gy) of r,u,v,p
    __device__ static G8<double> ld(const double2* G, int i) {
        G8<double> g;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            double2 a = __ldg(G + 4 * i + k);
            g.gx[k] = a.x; g.gy[k] = a.y;
        }
        return g;
    }
    __device__ static void st(double2* G, int i, const G8<double>& g) {
#pragma unroll
        for (int k = 0; k < 4; ++k) G[4 * i + k] = make_double2(g.gx[k], g.gy[k]);
    }
};
template <> struct GStore<float> {
    using type = float4;  // 2 x float4 per cell
    __device__ static G8<float> ld(const float4* G, int i) {
        float4 a = __ldg(G + 2 * i), b = __ldg(G + 2 * i + 1);
        G8<float> g;
        g.gx[0] = a.x; g.gy[0] = a.y; g.gx[1] = a.z; g.gy[1] = a.w;
        g.gx[2] = b.x; g.gy[2] = b.y; g.gx[3] = b.z; g.gy[3] = b.w;
        return g;
    }
    __device__ static void st(float4* G, int i, const G8<float>& g) {
        G[2 * i] = make_float4(g.gx[0], g.gy[0], g.gx[1], g.gy[1]);
        G[2 * i + 1] = make_float4(g.gx[2], g.gy[2], g.gx[3], g.gy[3]);
    }
};

// Flux-precision geometry: the solver stores these arrays as double (FP64
// mode) or float (FP32-flux mode), so no conversion is issued per use.
template <typename T> __device__ __forceinline__ T pick(double d, float f) {
    if constexpr (std::is_same<T, double>::value) return d;
    else return f;
}
template <typename T> __device__ __forceinline__ void ld_pair(const void* p, int i, T& x, T& y) {
    if constexpr (std::is_same<T, double>::value) {
        const double2 q = __ldg(static_cast<const double2*>(p) + i);
        x = q.x; y = q.y;
    } else {
        const float2 q = __ldg(static_cast<const float2*>(p) + i);
        x = q.x; y = q.y;
    }
}
template <typename T> __device__ __forceinline__ void ld_quad(const void* p, int i, T& x, T& y, T& z, T& w) {
    if constexpr (std::is_same<T, double>::value) {
        const double4_32a q = static_cast<const double4_32a*>(p)[i];
        x = q.x; y = q.y; z = q.z; w = q.w;
    } else {
        const float4 q = __ldg(static_cast<const float4*>(p) + i);
        x = q.x; y = q.y; z = q.z; w = q.w;
    }
}
template <typename T> __device__ __forceinline__ T ld_one(const void* p, int i) {
    return __ldg(static_cast<const T*>(p) + i);
}

// Face flux storage: double -> St; float -> float4.  Loaded as FP64 in the
// gather (exact widening on the integer pipe).
__device__ __forceinline__ void st_flux(St* ff, int f, const V4<double>& F) { st_state(ff, f, st_make(F.r, F.u, F.v, F.p)); }
__device__ __forceinline__ void st_flux(float4* ff, int f, const V4<float>& F) { ff[f] = make_float4(F.r, F.u, F.v, F.p); }
__device__ __forceinline__ St ld_flux(const St* ff, int f) { return ld_state(ff, f); }
__device__ __forceinline__ St ld_flux(const float4* ff, int f) {
    float4 a = __ldg(ff + f);
    return st_make(fvconv::f2d(a.x), fvconv::f2d(a.y), fvconv::f2d(a.z), fvconv::f2d(a.w));
}

// FP32-flux gather: the float face fluxes of a cell are summed in
// float-float (Knuth's TwoSum per addition, the rounding errors collected
// in a second float) on the FP32 pipe, and hi + lo is widened and added
// once in FP64.  Each addition is error-free and the error collector rounds
// at 2^-24 of the errors, so the sum is exact to about 2^-48 relative (the
// FP64 sum of the widened fluxes: 2^-53).  With LAM the per-face wave-speed
// terms of the local time step (stored as floats) are summed in FP32.
__device__ __forceinline__ void two_sum_acc(float& hi, float& lo, float x) {
    const float s = hi + x;
    const float bp = s - hi;
    lo += (hi - (s - bp)) + (x - bp);
    hi = s;
}
__device__ __forceinline__ float4 flipf(const float4& F, int neg) {
    const unsigned m = (unsigned)(neg & 1) << 31;
    return make_float4(__uint_as_float(__float_as_uint(F.x) ^ m), __uint_as_float(__float_as_uint(F.y) ^ m),
                       __uint_as_float(__float_as_uint(F.z) ^ m), __uint_as_float(__float_as_uint(F.w) ^ m));
}
template <bool LAM>
__device__ __forceinline__ St gather32(const float4* __restrict__ ff, const float* __restrict__ lamf_face,
                                       const int* __restrict__ cf, int e0, int e1, float& lam) {
    const int ent0 = cf[e0];
    float4 h = flipf(__ldg(ff + (ent0 >> 1)), ent0);
    float4 l = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    if (LAM) lam = __ldg(lamf_face + (ent0 >> 1));
    for (int e = e0 + 1; e < e1; ++e) {
        const int ent = cf[e];
        const int f = ent >> 1;
        const float4 q = flipf(__ldg(ff + f), ent);
        two_sum_acc(h.x, l.x, q.x);
        two_sum_acc(h.y, l.y, q.y);
        two_sum_acc(h.z, l.z, q.z);
        two_sum_acc(h.w, l.w, q.w);
        if (LAM) lam += __ldg(lamf_face + f);
    }
    return st_make(fvconv::f2d(h.x) + fvconv::f2d(l.x), fvconv::f2d(h.y) + fvconv::f2d(l.y),
                   fvconv::f2d(h.z) + fvconv::f2d(l.z), fvconv::f2d(h.w) + fvconv::f2d(l.w));
}

// ---------------------------------------------------------------------------
// Primitive-input physics
// ---------------------------------------------------------------------------
template <typename T>
__device__ __forceinline__ V4<T> phys_flux_p(const V4<T>& w, T E, T Vn, T nx, T ny) {
    return {w.r * Vn, w.r * w.u * Vn + w.p * nx, w.r * w.v * Vn + w.p * ny, (E + w.p) * Vn};
}

// Rusanov on primitive inputs (RusanovFlux.h:33-43 with cached primitives).
template <typename T>
__device__ __forceinline__ V4<T> rusanov_p(const V4<T>& L, const V4<T>& R, T nx, T ny, T g, T igm1) {
    T cL = tsqrt<T>(g * L.p / L.r), cR = tsqrt<T>(g * R.p / R.r);
    T VnL = L.u * nx + L.v * ny, VnR = R.u * nx + R.v * ny;
    T EL = L.p * igm1 + T(0.5) * L.r * (L.u * L.u + L.v * L.v);
    T ER = R.p * igm1 + T(0.5) * R.r * (R.u * R.u + R.v * R.v);
    T Smax = fmax(fabs(VnL) + cL, fabs(VnR) + cR);
    V4<T> FL = phys_flux_p(L, EL, VnL, nx, ny), FR = phys_flux_p(R, ER, VnR, nx, ny);
    T h = T(0.5) * Smax;
    return {T(0.5) * (FL.r + FR.r) - h * (R.r - L.r),
            T(0.5) * (FL.u + FR.u) - h * (R.r * R.u - L.r * L.u),
            T(0.5) * (FL.v + FR.v) - h * (R.r * R.v - L.r * L.v),
            T(0.5) * (FL.p + FR.p) - h * (ER - EL)};
}

// HLLC on primitive inputs (HllcFlux.h:35-76), rearranged for the FP64
// pipe: the sound speeds come from one reciprocal square root each
// (c = g p / sqrt(g p rho)), the energy only of the upwind side that the
// flux uses, and with q = 1/(S_K - S*) the star factor is
// rho_K (S_K - Vn_K) q and the star energy needs no 1/rho_K (below).
template <typename T> __device__ __forceinline__ T trsqrt(T x);
template <> __device__ __forceinline__ double trsqrt<double>(double x) { return rsqrt(x); }
template <> __device__ __forceinline__ float trsqrt<float>(float x) { return rsqrtf(x); }

// a / b where only the quotient's value matters to within an ulp (the
// limiter, the local time step): FP64 as a times fvconv::rcp_nr3(b), which
// issues fewer FP64-pipe instructions on this part than the correctly
// rounded division or the built-in reciprocal (ncu counts per cell); FP32
// as the division.  HLLC keeps the built-in reciprocal, which measured
// fewer there.
template <typename T> __device__ __forceinline__ T tdiv(T a, T b) { return a / b; }
template <> __device__ __forceinline__ double tdiv<double>(double a, double b) { return a * fvconv::rcp_nr3(b); }

template <typename T>
__device__ __forceinline__ V4<T> hllc_p(const V4<T>& L, const V4<T>& R, T nx, T ny, T g, T igm1) {
    const T gpL = g * L.p, gpR = g * R.p;
    T cL = gpL * trsqrt<T>(gpL * L.r), cR = gpR * trsqrt<T>(gpR * R.r);
    T VnL = L.u * nx + L.v * ny, VnR = R.u * nx + R.v * ny;
    T SL = fmin(VnL - cL, VnR - cR), SR = fmax(VnL + cL, VnR + cR);
    if (SL >= T(0)) return phys_flux_p(L, L.p * igm1 + T(0.5) * L.r * (L.u * L.u + L.v * L.v), VnL, nx, ny);
    if (SR <= T(0)) return phys_flux_p(R, R.p * igm1 + T(0.5) * R.r * (R.u * R.u + R.v * R.v), VnR, nx, ny);
    const T dL = SL - VnL, dR = SR - VnR;
    T mL = L.r * dL, mR = R.r * dR;
    // S* = num / den with den = m_L - m_R < 0 (S_L < Vn_L and S_R > Vn_R),
    // so the side is known before any division: S* >= 0 <=> num <= 0.  Both
    // S* and q = 1 / (S_K - S*) = den / (S_K den - num) then come from one
    // reciprocal of den (S_K den - num), which issues fewer FP64-pipe
    // instructions on this part than two.
    const T num = R.p - L.p + mL * VnL - mR * VnR, den = mL - mR;
    bool left = num <= T(0);
    T SK = left ? SL : SR, VnK = left ? VnL : VnR;
    T mK = left ? mL : mR, dK = left ? dL : dR;
    V4<T> K = left ? L : R;
    const T EK = K.p * igm1 + T(0.5) * K.r * (K.u * K.u + K.v * K.v);
    const T t = SK * den - num;
    const T rr = T(1) / (den * t);
    const T Ss = num * (t * rr);
    T q = den * (den * rr);
    T fac = mK * q;
    T VtK = -K.u * ny + K.v * nx;
    T mn = fac * Ss, mt = fac * VtK;
    // E* = rho*_K [E_K / rho_K + (S* - Vn_K)(S* + p_K / (rho_K (S_K - Vn_K)))]
    // with rho*_K = m_K q: the 1/rho_K cancels, leaving
    // E* = q [(S_K - Vn_K) E_K + (S* - Vn_K)(m_K S* + p_K)].
    T Es = q * (dK * EK + (Ss - VnK) * (mK * Ss + K.p));
    V4<T> FK = phys_flux_p(K, EK, VnK, nx, ny);
    return {FK.r + SK * (fac - K.r),
            FK.u + SK * ((mn * nx - mt * ny) - K.r * K.u),
            FK.v + SK * ((mn * ny + mt * nx) - K.r * K.v),
            FK.p + SK * (Es - EK)};
}

template <typename T>
__device__ __forceinline__ V4<T> prim_of(const St& s, T g) {
    T r = (T)s.r;
    T u = (T)(s.ru / s.r), v = (T)(s.rv / s.r);
    T p = (T)((g - 1.0) * (s.E - 0.5 * s.r * ((s.ru / s.r) * (s.ru / s.r) + (s.rv / s.r) * (s.rv / s.r))));
    return {r, u, v, p};
}

// Primitive freestream of a farfield patch from its conserved state.
template <typename T>
__device__ __forceinline__ V4<T> fs_prim(const double* st, T g) {
    T rf = (T)st[0];
    T uf = (T)(st[1] / st[0]), vf = (T)(st[2] / st[0]);
    T pf = (T)((g - 1.0) * (st[3] - 0.5 * st[0] * ((st[1] / st[0]) * (st[1] / st[0]) + (st[2] / st[0]) * (st[2] / st[0]))));
    return {rf, uf, vf, pf};
}

// Ghost state in primitive form from the patch kind, the interior state w,
// the primitive freestream fsp (farfield kinds) and the wall velocity
// (no-slip).  Shared by the residual kernels and, on dual numbers, by the
// discrete adjoint's linearisation.
template <typename T>
__device__ __forceinline__ V4<T> ghost_core(int t, const V4<T>& w, T nx, T ny, T g, const V4<T>& fsp, T wall_u,
                                            T wall_v) {
    if (t == BC_OUTFLOW) return w;
    if (t == BC_FARFIELD || t == BC_CHAR) {
        const T rf = fsp.r, uf = fsp.u, vf = fsp.v, pf = fsp.p;
        if (t == BC_FARFIELD) return {rf, uf, vf, pf};
        T ci = tsqrt<T>(g * w.p / w.r), cf = tsqrt<T>(g * pf / rf);
        T vni = w.u * nx + w.v * ny, vnf = uf * nx + vf * ny;
        if (vnf <= -cf) return {rf, uf, vf, pf};
        if (vni >= ci) return w;
        T k = T(2) / (g - T(1));
        T Rp = vni + k * ci, Rm = vnf - k * cf;
        T vnb = T(0.5) * (Rp + Rm);
        T cb = T(0.25) * (g - T(1)) * (Rp - Rm);
        T s, ut, vt;
        if (vnb > T(0)) { s = w.p / tpow<T>(w.r, g); ut = w.u - vni * nx; vt = w.v - vni * ny; }
        else { s = pf / tpow<T>(rf, g); ut = uf - vnf * nx; vt = vf - vnf * ny; }
        T rb = tpow<T>(cb * cb / (g * s), T(1) / (g - T(1)));
        T pb = rb * cb * cb / g;
        return {rb, ut + vnb * nx, vt + vnb * ny, pb};
    }
    if (t == BC_NOSLIP) return {w.r, T(2) * wall_u - w.u, T(2) * wall_v - w.v, w.p};
    T Vn = w.u * nx + w.v * ny;
    return {w.r, w.u - T(2) * Vn * nx, w.v - T(2) * Vn * ny, w.p};
}

// Ghost state in primitive form (EulerFVMSolver::ghost_state,
// src/EulerFVMSolver.cpp:174-193, plus the characteristic farfield).
// fs, when given, replaces the patch's freestream state (batched solves:
// one freestream per instance).
template <typename T>
__device__ __forceinline__ V4<T> ghost_prim(const BCTable& bc, int patch, const V4<T>& w, T nx, T ny, T g,
                                            const double* fs = nullptr) {
    const int t = bc.type[patch];
    V4<T> fsp = {T(0), T(0), T(0), T(0)};
    if (t == BC_FARFIELD || t == BC_CHAR) fsp = fs_prim<T>(fs ? fs : bc.st[patch], g);
    T wu = T(0), wv = T(0);
    if (t == BC_NOSLIP) { wu = (T)bc.wall_u[patch]; wv = (T)bc.wall_v[patch]; }
    return ghost_core<T>(t, w, nx, ny, g, fsp, wu, wv);
}

using fvgb::O2Args;

// Face normal, length and CFL length in flux precision.
template <typename T> __device__ __forceinline__ void face_geom(const O2Args& a, int f, T& nx, T& ny, T& ar, T& len) {
    if constexpr (std::is_same<T, double>::value) {
        const double4_32a q = a.m.fgeom[f];
        nx = q.x; ny = q.y; ar = q.z; len = q.w;
    } else {
        const float4 q = __ldg(a.fgeom32 + f);
        nx = q.x; ny = q.y; ar = q.z; len = q.w;
    }
}

// Order-preserving integer key of an IEEE value (negative values have their
// magnitude bits flipped), so that integer compares -- on the integer pipe,
// not the scarce FP64 pipe -- order values like the floating-point compare
// (NaNs excepted).  val() inverts key().
template <typename T> struct OKey;
template <> struct OKey<double> {
    using I = long long;
    __device__ static I bits(double x) { return __double_as_longlong(x); }
    __device__ static double from_bits(I b) { return __longlong_as_double(b); }
    __device__ static I sign_bit() { return (I)0x8000000000000000ULL; }
    __device__ static I one_exp() { return (I)1 << 52; }  // +1 in the exponent field
    __device__ static I key(double x) { I b = __double_as_longlong(x); return b ^ ((b >> 63) & 0x7fffffffffffffffLL); }
    __device__ static double val(I k) { return __longlong_as_double(k ^ ((k >> 63) & 0x7fffffffffffffffLL)); }
};
template <> struct OKey<float> {
    using I = int;
    __device__ static I bits(float x) { return __float_as_int(x); }
    __device__ static float from_bits(I b) { return __int_as_float(b); }
    __device__ static I sign_bit() { return (I)0x80000000u; }
    __device__ static I one_exp() { return (I)1 << 23; }
    __device__ static I key(float x) { I b = __float_as_int(x); return b ^ ((b >> 31) & 0x7fffffff); }
    __device__ static float val(I k) { return __int_as_float(k ^ ((k >> 31) & 0x7fffffff)); }
};

// ---------------------------------------------------------------------------
// Register caps: FP32 mode is latency bound (<= 64 registers, 32 warps per
// SM); FP64 mode <= 128 (16 warps keep the FP64 pipe fed).
template <typename T, int GRAD, int LIM>
__global__ void __launch_bounds__(fvgb::kMaxBlock, sizeof(T) == 4 ? 2 : 1) k_grad(const O2Args a) {
    using WS = WStore<T>;
    using WT = typename WS::type;
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= a.m.n_cells) return;
    // Batched solves: converged instances are frozen; each instance has
    // its own freestream.
    const double* fs = nullptr;
    if (a.cell_inst) {
        const int inst = a.cell_inst[c];
        if (a.active && !a.active[inst]) return;
        fs = a.inst_fs + 4 * inst;
    }
    const WT* W = static_cast<const WT*>(a.W);
    const T g = pick<T>(a.gamma, a.gamma32);
    const V4<T> wc = WS::ld(W, c);
    const T* wcv = &wc.r;
    using OK = OKey<T>;
    using I = typename OK::I;
    T gx[4] = {0, 0, 0, 0}, gy[4] = {0, 0, 0, 0}, dmax[4] = {0, 0, 0, 0}, dmin[4] = {0, 0, 0, 0};
    // Neighbour max/min on the integer pipe: order-preserving integer keys of
    // the values, starting from the cell's own value (so that
    // max_j W_j - W_c equals the max over the differences, including 0,
    // bit for bit).
    I kmax[4], kmin[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) kmax[k] = kmin[k] = OK::key(wcv[k]);
    const int e0 = a.m.cf_off[c], e1 = a.m.cf_off[c + 1];
    for (int e = e0; e < e1; ++e) {
        const int nb = a.cnb[e];
        V4<T> wn;
        if (nb >= 0) {
            wn = WS::ld(W, nb);
        } else {
            const int f = -1 - nb;
            T nx, ny, ar, len;
            face_geom<T>(a, f, nx, ny, ar, len);
            V4<T> gh = ghost_prim<T>(a.bc, a.m.fpatch[f], wc, nx, ny, g, fs);
            wn = {T(0.5) * (wc.r + gh.r), T(0.5) * (wc.u + gh.u), T(0.5) * (wc.v + gh.v), T(0.5) * (wc.p + gh.p)};
        }
        const T* wnv = &wn.r;
        if (GRAD == 0) {
            // sum_j a_j (W_j - W_c) = sum_j a_j W_j - (sum_j a_j) W_c; the
            // weight sums are per-cell geometry (lsq_sum).
            T ax, ay;
            ld_pair<T>(a.lsq, e, ax, ay);
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const I kk = OK::key(wnv[k]);
                kmax[k] = kmax[k] < kk ? kk : kmax[k];
                kmin[k] = kk < kmin[k] ? kk : kmin[k];
                gx[k] += ax * wnv[k];
                gy[k] += ay * wnv[k];
            }
        } else {
            T ax, ay, wgt, unused;
            ld_quad<T>(a.gg, e, ax, ay, wgt, unused);
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                T d = wnv[k] - wcv[k];
                dmax[k] = fmax(dmax[k], d);
                dmin[k] = fmin(dmin[k], d);
                T phif = wgt * wcv[k] + (T(1) - wgt) * wnv[k];
                gx[k] += ax * phif;
                gy[k] += ay * phif;
            }
        }
    }
    if (GRAD == 0) {
        T sx, sy;
        ld_pair<T>(a.lsq_sum, c, sx, sy);
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            gx[k] -= sx * wcv[k];
            gy[k] -= sy * wcv[k];
            dmax[k] = OK::val(kmax[k]) - wcv[k];
            dmin[k] = OK::val(kmin[k]) - wcv[k];
        }
    }
    if constexpr (sizeof(T) == 8) {
        if (a.lim_gu) {
#pragma unroll
            for (int k = 0; k < 4; ++k) a.lim_gu[4 * c + k] = make_double2(gx[k], gy[k]);
            if (LIM == 0)
                for (int k = 0; k < 4; ++k) a.lim_psi[4 * c + k] = 1.0;
        }
    }
    // FP64 with a limiter: k_face reconstructs from the per-entry
    // increments and the per-cell limiter values (O2Args::d2); the limited
    // gradients are not stored.
    bool dpath = false;
    if constexpr (sizeof(T) == 8) dpath = LIM != 0 && a.d2 != nullptr;
    if (LIM != 0 && a.psi_mode == 2) {
        // frozen limiter: the values captured earlier (psi = 1 scales exactly)
        const T* pb = static_cast<const T*>(a.psi_buf) + 4 * (size_t)c;
        if constexpr (sizeof(T) == 8) {
            if (dpath) {
                for (int e = e0; e < e1; ++e) {
                    T rx, ry;
                    ld_pair<T>(a.erf, e, rx, ry);
                    st_state(a.d2, e, st_make(gx[0] * rx + gy[0] * ry, gx[1] * rx + gy[1] * ry,
                                              gx[2] * rx + gy[2] * ry, gx[3] * rx + gy[3] * ry));
                }
                st_state(a.psi4, c, st_make(pb[0], pb[1], pb[2], pb[3]));
                return;
            }
        }
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const T psi = pb[k];
            if constexpr (sizeof(T) == 8) {
                if (a.lim_psi) a.lim_psi[4 * c + k] = psi;
            }
            gx[k] *= psi;
            gy[k] *= psi;
        }
    } else if (LIM != 0) {
        const T eps2 = LIM == 2 ? ld_one<T>(a.eps2, c) : T(0);
        // Per face f the limiter value is psi_f = phi(D1, D2_f) with D2_f the
        // unlimited extrapolation to the face and D1 = dmax (D2_f > 0) or
        // dmin (D2_f < 0).  With D1 fixed per sign, phi only limits
        // (phi < 1) where |D1| < 2|D2| (Venkatakrishnan) or |D1| < |D2|
        // (Barth-Jespersen), and there it strictly decreases in |D2|; so
        // min(1, min_f psi_f) = min(1, phi(dmax, max D2 > 0),
        // phi(dmin, min D2 < 0)).  Per face only D2 is formed; its extremes
        // are tracked as integer maxima of the bit patterns (positive side:
        // bits of D2; negative side: bits of -D2), off the FP64 pipe.
        I pmax[4] = {0, 0, 0, 0}, nmax[4] = {0, 0, 0, 0};
        const I sign = OK::sign_bit();
        for (int e = e0; e < e1; ++e) {
            T rx, ry;
            ld_pair<T>(a.erf, e, rx, ry);
            T d2v[4];
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                d2v[k] = gx[k] * rx + gy[k] * ry;
                const I b = OK::bits(d2v[k]);
                pmax[k] = pmax[k] < b ? b : pmax[k];
                const I bn = b ^ sign;
                nmax[k] = nmax[k] < bn ? bn : nmax[k];
            }
            if constexpr (sizeof(T) == 8) {
                if (dpath) st_state(a.d2, e, st_make(d2v[0], d2v[1], d2v[2], d2v[3]));
            }
        }
        T psiv[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            T nmin = T(1), dmn = T(1);
            bool lim = false;
#pragma unroll
            for (int side = 0; side < 2; ++side) {
                const I yb = side == 0 ? pmax[k] : nmax[k];
                if (yb <= 0) continue;                       // no face with D2 of this sign
                const T y = OK::from_bits(yb);               // |D2| extreme, > 0
                const T d1 = side == 0 ? dmax[k] : -dmin[k];  // |D1| >= 0
                // phi(d1, y) < 1 only where d1 < 2y (Venkatakrishnan: the
                // eps^2 terms cancel in num < den) or d1 < y (Barth-
                // Jespersen); for d1 >= 0 and y > 0 that compare is an
                // integer compare of the bit patterns, so a side that cannot
                // limit costs no FP64 instruction.
                {
                    using U = typename std::make_unsigned<I>::type;
                    const I bound = LIM == 1 ? yb : (I)((U)yb + (U)OK::one_exp());
                    if (!(OK::bits(d1) < bound)) continue;
                }
                T num, den;
                if (LIM == 1) {
                    num = d1;
                    den = y;
                } else {
                    // (d1^2 + eps^2 + 2 d1 y) / (d1^2 + 2 y^2 + d1 y + eps^2)
                    const T p = d1 * y;
                    const T q = d1 * d1 + eps2;
                    num = q + T(2) * p;
                    // 2y by incrementing the exponent of y's bit pattern
                    // (integer pipe; y > 0: exact for normal y, infinity
                    // past the largest binade as 2y would be; a subnormal
                    // y gives a value below twice the smallest normal, as
                    // 2y is, which only scales an already negligible 2y^2)
                    using U = typename std::make_unsigned<I>::type;  // wraps, never overflows
                    const T y2 = OK::from_bits((I)((U)yb + (U)OK::one_exp()));
                    den = y2 * y + (q + p);
                }
                if (num * dmn < nmin * den) { nmin = num; dmn = den; lim = true; }
            }
            // psi = 1 needs no division or scaling
            const T psi = lim ? tdiv<T>(nmin, dmn) : T(1);
            if constexpr (sizeof(T) == 8) {
                if (a.lim_psi) a.lim_psi[4 * c + k] = psi;
            }
            if (a.psi_mode == 1) static_cast<T*>(a.psi_buf)[4 * (size_t)c + k] = psi;
            psiv[k] = psi;
            if (lim && !dpath) {
                gx[k] *= psi;
                gy[k] *= psi;
            }
        }
        if constexpr (sizeof(T) == 8) {
            if (dpath) {
                st_state(a.psi4, c, st_make(psiv[0], psiv[1], psiv[2], psiv[3]));
                return;
            }
        }
    }
    G8<T> out;
#pragma unroll
    for (int k = 0; k < 4; ++k) { out.gx[k] = gx[k]; out.gy[k] = gy[k]; }
    GStore<T>::st(static_cast<typename GStore<T>::type*>(a.G), c, out);
}

template <typename T>
__device__ __forceinline__ V4<T> recon(const V4<T>& w, const G8<T>& g, T rx, T ry) {
    // w + gx rx + gy ry as two multiply-adds (contracted to FMA)
    V4<T> o = {g.gx[0] * rx + (g.gy[0] * ry + w.r), g.gx[1] * rx + (g.gy[1] * ry + w.u),
               g.gx[2] * rx + (g.gy[2] * ry + w.v), g.gx[3] * rx + (g.gy[3] * ry + w.p)};
    // Positivity fallback; "x > 0" tested on the integer pipe (sign bit clear
    // and not +0).
    if (OKey<T>::bits(o.r) <= 0 || OKey<T>::bits(o.p) <= 0) return w;
    return o;
}

// w + psi * inc (the limited increment to the face, one multiply-add per
// variable), with recon's positivity fallback.
__device__ __forceinline__ V4<double> recon_inc(const V4<double>& w, const St& psi, const St& inc) {
    const V4<double> o = {psi.r * inc.r + w.r, psi.ru * inc.ru + w.u, psi.rv * inc.rv + w.v, psi.E * inc.E + w.p};
    if (OKey<double>::bits(o.r) <= 0 || OKey<double>::bits(o.p) <= 0) return w;
    return o;
}

template <typename T, int FLUX>
__device__ __forceinline__ V4<T> num_flux_p(const V4<T>& L, const V4<T>& R, T nx, T ny, T g, T igm1, double tol,
                                            int maxit) {
    if constexpr (FLUX == FLUX_HLLC) return hllc_p<T>(L, R, nx, ny, g, igm1);
    else if constexpr (FLUX == FLUX_EXACT) {
        St UL = from_primitive((double)L.r, (double)L.u, (double)L.v, (double)L.p, (double)g);
        St UR = from_primitive((double)R.r, (double)R.u, (double)R.v, (double)R.p, (double)g);
        St F = exact_riemann(UL, UR, (double)nx, (double)ny, (double)g, tol, maxit);
        return {(T)F.r, (T)F.ru, (T)F.rv, (T)F.E};
    } else return rusanov_p<T>(L, R, nx, ny, g, igm1);
}

// DT: 0 = no time step this stage, 1 = global (atomicMin), 2 = local (per face).
template <typename T, int FLUX, int ORDER, int DT>
__global__ void __launch_bounds__(fvgb::kMaxBlock) k_face(const O2Args a) {
    using WS = WStore<T>;
    using WT = typename WS::type;
    using FT = typename std::conditional<std::is_same<T, double>::value, St, float4>::type;
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    double cand = DBL_MAX;
    // Batched solves (local dt only): faces of converged instances are skipped.
    const bool live = f < a.m.n_faces && (!a.active || a.active[a.cell_inst[a.m.fl[f]]]);
    if (live) {
        const WT* W = static_cast<const WT*>(a.W);
        const T g = pick<T>(a.gamma, a.gamma32), igm1 = pick<T>(a.igm1, a.igm1_32);
        const int L = a.m.fl[f], R = a.m.fr[f];
        const double* fs = a.cell_inst ? a.inst_fs + 4 * a.cell_inst[L] : nullptr;
        T nx, ny, ar, len;
        face_geom<T>(a, f, nx, ny, ar, len);
        V4<T> wl = WS::ld(W, L), wr;
        const V4<T> wlc = wl;
        bool dpath = false;
        if constexpr (sizeof(T) == 8) dpath = ORDER == 2 && a.d2 != nullptr;
        if (dpath) {
            if constexpr (sizeof(T) == 8) {
                const int2 ee = __ldg(a.fe + f);
                wl = recon_inc(wl, ld_state(a.psi4, L), ld_state(a.d2, ee.x));
                if (R >= 0) wr = recon_inc(WS::ld(W, R), ld_state(a.psi4, R), ld_state(a.d2, ee.y));
            }
        } else if (ORDER == 2) {
            T rxl, ryl, rxr, ryr;
            ld_quad<T>(a.frf, f, rxl, ryl, rxr, ryr);
            const G8<T> gl = GStore<T>::ld(static_cast<const typename GStore<T>::type*>(a.G), L);
            wl = recon<T>(wl, gl, rxl, ryl);
            if (R >= 0) {
                const G8<T> gr = GStore<T>::ld(static_cast<const typename GStore<T>::type*>(a.G), R);
                wr = recon<T>(WS::ld(W, R), gr, rxr, ryr);
            }
        } else if (R >= 0) {
            wr = WS::ld(W, R);
        }
        if (R < 0) wr = ghost_prim<T>(a.bc, a.m.fpatch[f], wl, nx, ny, g, fs);
        const V4<T> F = num_flux_p<T, FLUX>(wl, wr, nx, ny, g, igm1, a.exact_tol, a.exact_max_iter);
        st_flux(static_cast<FT*>(a.ff), f, V4<T>{ar * F.r, ar * F.u, ar * F.v, ar * F.p});
        if (DT != 0) {
            // compute_dt's per-face candidate from cell-centred states
            // (src/EulerFVMSolver.cpp:140-160).  FP32-flux mode forms the
            // wave speed in FP32 (the sound speed is stored in FP32 there):
            // local dt keeps lambda * A as a float for k_update's FP32 sum;
            // the global-dt candidate is widened exactly and formed in FP64.
            const T* cs = static_cast<const T*>(a.cs);
            T Smax = fabs(wlc.u * nx + wlc.v * ny) + cs[L];
            if (R >= 0) {
                const V4<T> wrc = WS::ld(W, R);
                Smax = rmax(Smax, fabs(wrc.u * nx + wrc.v * ny) + cs[R]);
            }
            if constexpr (std::is_same<T, double>::value) {
                if (DT == 2) a.dtf[f] = Smax * ar;
                else cand = a.ctl->cfl * len / Smax;
            } else {
                if (DT == 2) reinterpret_cast<float*>(a.dtf)[f] = Smax * ar;
                else cand = a.ctl->cfl * fvconv::f2d(len) / fvconv::f2d(Smax);
            }
        }
    }
    if (DT == 1) {
        __shared__ double smin[fvgb::kMaxBlock / 32];
        cand = warp_min(cand);
        if ((threadIdx.x & 31) == 0) smin[threadIdx.x >> 5] = cand;
        __syncthreads();
        if (threadIdx.x == 0) {
            double v = smin[0];
            for (int w = 1; w < (int)(blockDim.x >> 5); ++w) v = fmin(v, smin[w]);
            atomicMin(&a.ctl->dt_bits, (unsigned long long)__double_as_longlong(v));
        }
    }
}

// FP32-flux mode: the primitive copy and the sound speed only feed FP32
// arithmetic (fluxes, the wave speed of the time step), so they are derived
// in FP32 from the state rounded on the integer pipe; nothing here issues
// on the FP64 pipe.  Shared by the update and by the refresh after a state
// upload, so both leave the same W.
__device__ __forceinline__ V4<float> prim32(const St& un, float gf, float& cs) {
    const float rf = fvconv::d2f(un.r), irf = 1.0f / rf;
    const float uf = fvconv::d2f(un.ru) * irf, vf = fvconv::d2f(un.rv) * irf;
    const float pf = (gf - 1.0f) * (fvconv::d2f(un.E) - 0.5f * rf * (uf * uf + vf * vf));
    cs = sqrtf(gf * pf * irf);
    return {rf, uf, vf, pf};
}

// STAGE: 0..NST-1; NST: 1 (forward Euler) or 3 (SSP-RK3); DT: 1 global, 2 local.
template <typename T, int STAGE, int NST, int DT>
__global__ void __launch_bounds__(fvgb::kMaxBlock) k_update(const O2Args a) {
    using FT = typename std::conditional<std::is_same<T, double>::value, St, float4>::type;
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
    if (c < a.m.n_cells && (!a.active || a.active[a.cell_inst[c]])) {
        const FT* ff = static_cast<const FT*>(a.ff);
        const int e0 = a.m.cf_off[c], e1 = a.m.cf_off[c + 1];
        St R;
        double lam = 0.0;
        float lamf = 0.0f;
        if constexpr (std::is_same<T, float>::value) {
            R = gather32<STAGE == 0 && DT == 2>(ff, reinterpret_cast<const float*>(a.dtf), a.m.cf, e0, e1, lamf);
        } else {
            // Every cell has faces: the sum starts from the first signed flux
            // instead of 0 + flux (one FP64 add per component less; only the
            // sign of an exactly-zero sum can differ, and u + dt * (+-0) = u).
            const int ent0 = a.m.cf[e0];
            R = flip_if(ld_flux(ff, ent0 >> 1), ent0);
            if (STAGE == 0 && DT == 2) lam = a.dtf[ent0 >> 1];
            for (int e = e0 + 1; e < e1; ++e) {
                const int ent = a.m.cf[e];
                const int f = ent >> 1;
                R += flip_if(ld_flux(ff, f), ent);
                if (STAGE == 0 && DT == 2) lam += a.dtf[f];
            }
        }
        if (a.forcing) R += ld_state(a.forcing, c);
        double dtv;
        if (STAGE == 0) {
            // Local: dt_i = cfl V_i / sum_f lambda_f A_f, so dt_i / V_i = cfl / sum
            // (FP32-flux mode: in FP32; the step size only sets the path to the
            // steady state); global: the min over faces, divided by the volume.
            if (DT == 2) {
                if constexpr (std::is_same<T, float>::value) dtv = fvconv::f2d(fvconv::d2f(a.ctl->cfl) / lamf);
                else dtv = tdiv<double>(a.ctl->cfl, lam);
            } else {
                dtv = __longlong_as_double((long long)a.ctl->dt_bits) / a.m.vol[c];
            }
            if (NST > 1) a.dtv[c] = dtv;
            s0 = R.r * R.r; s1 = R.ru * R.ru; s2 = R.rv * R.rv; s3 = R.E * R.E;
            if (a.r2) {
                double4_32a q;
                q.x = s0; q.y = s1; q.z = s2; q.w = s3;
                a.r2[c] = q;
            }
        } else {
            dtv = a.dtv[c];
        }
        const St u = ld_state(a.U, c);
        const St e = u + dtv * R;
        St un;
        if (NST == 1) un = e;
        else if (STAGE == 0) { st_state(a.U0, c, u); un = e; }
        else if (STAGE == 1) un = 0.75 * ld_state(a.U0, c) + 0.25 * e;
        else un = (1.0 / 3.0) * ld_state(a.U0, c) + (2.0 / 3.0) * e;
        st_state(a.U, c, un);
        const double g = a.gamma;
        if constexpr (std::is_same<T, float>::value) {
            float cs;
            WStore<T>::st(static_cast<typename WStore<T>::type*>(a.W), c, prim32(un, a.gamma32, cs));
            if (STAGE == NST - 1) static_cast<float*>(a.cs)[c] = cs;
        } else {
            const double ir = fvconv::rcp_nr3(un.r);  // same as k_prim / k_update
            const double uu = un.ru * ir, vv = un.rv * ir;
            const double p = (g - 1.0) * (un.E - 0.5 * un.r * (uu * uu + vv * vv));
            WStore<T>::st(static_cast<typename WStore<T>::type*>(a.W), c, V4<T>{un.r, uu, vv, p});
            if (STAGE == NST - 1) static_cast<double*>(a.cs)[c] = sqrt(g * p * ir);
        }
    }
    // Batched solves reduce per instance instead (k_batch_norms); a.r2 is
    // uniform over the grid, so the block-wide reduction is all-or-nothing.
    if (STAGE == 0 && !a.r2) finish_norms(s0, s1, s2, s3, a.ctl, a.partials, a.hist, a.hist_cap);
}

// Residual only (multigrid restriction): the same signed gather as
// k_update, plus the forcing term, stored per cell.
template <typename T>
__global__ void __launch_bounds__(fvgb::kMaxBlock) k_residual(const O2Args a) {
    using FT = typename std::conditional<std::is_same<T, double>::value, St, float4>::type;
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= a.m.n_cells) return;
    const FT* ff = static_cast<const FT*>(a.ff);
    const int e0 = a.m.cf_off[c], e1 = a.m.cf_off[c + 1];
    St R;
    if constexpr (std::is_same<T, float>::value) {
        float unused;
        R = gather32<false>(ff, nullptr, a.m.cf, e0, e1, unused);
    } else {
        const int ent0 = a.m.cf[e0];
        R = flip_if(ld_flux(ff, ent0 >> 1), ent0);
        for (int e = e0 + 1; e < e1; ++e) {
            const int ent = a.m.cf[e];
            R += flip_if(ld_flux(ff, ent >> 1), ent);
        }
    }
    if (a.forcing) R += ld_state(a.forcing, c);
    st_state(a.resid, c, R);
}

// Per-instance residual norms of a batched solve: one block per instance
// folds the instance's cells (contiguous in device order) in a fixed
// order, records the norms and the iteration count, and freezes the
// instance once its density norm is below the tolerance.
static __global__ void __launch_bounds__(256) k_batch_norms(const O2Args a, const int* __restrict__ inst_off,
                                                      double* __restrict__ inst_norms, int* __restrict__ inst_iter,
                                                      int* __restrict__ active, double tol) {
    const int i = blockIdx.x;
    if (!active[i]) return;
    double t[4] = {0.0, 0.0, 0.0, 0.0};
    for (int c = inst_off[i] + threadIdx.x; c < inst_off[i + 1]; c += blockDim.x) {
        const double4_32a q = a.r2[c];
        t[0] += q.x; t[1] += q.y; t[2] += q.z; t[3] += q.w;
    }
    __shared__ double red[8][4];
#pragma unroll
    for (int k = 0; k < 4; ++k) t[k] = warp_sum(t[k]);
    if ((threadIdx.x & 31) == 0)
        for (int k = 0; k < 4; ++k) red[threadIdx.x >> 5][k] = t[k];
    __syncthreads();
    if (threadIdx.x == 0) {
        double n[4];
        for (int k = 0; k < 4; ++k) {
            double v = 0.0;
            for (int w = 0; w < 8; ++w) v += red[w][k];
            n[k] = sqrt(v);
            inst_norms[4 * i + k] = n[k];
        }
        inst_iter[i] += 1;
        if (n[0] < tol || !isfinite(n[0])) active[i] = 0;
    }
}

// Primitive copy + sound speed from U (after construction / set_field).
template <typename T>
__global__ void __launch_bounds__(fvgb::kCellBlock) k_prim(const O2Args a) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= a.m.n_cells) return;
    const St un = ld_state(a.U, c);
    const double g = a.gamma;
    const double ir = fvconv::rcp_nr3(un.r);  // same as k_prim / k_update
    const double uu = un.ru * ir, vv = un.rv * ir;
    const double p = (g - 1.0) * (un.E - 0.5 * un.r * (uu * uu + vv * vv));
    if constexpr (std::is_same<T, float>::value) {
        float cs;
        WStore<T>::st(static_cast<typename WStore<T>::type*>(a.W), c, prim32(un, a.gamma32, cs));
        static_cast<float*>(a.cs)[c] = cs;
    } else {
        WStore<T>::st(static_cast<typename WStore<T>::type*>(a.W), c, V4<T>{(T)un.r, (T)uu, (T)vv, (T)p});
        static_cast<double*>(a.cs)[c] = sqrt(g * p * ir);
    }
}

}  // namespace FV_KNS
