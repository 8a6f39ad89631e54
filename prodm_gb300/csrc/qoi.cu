// GE quantities of interest on the device (sm_103a): values and pointwise
// error estimates for the QoI-bounded retrieval drivers.
//
// Values: V_TOT = |V|, T = P / (D R), C = sqrt(gamma R T), Mach = V_TOT / C,
// PT = P (1 + (gamma - 1) / 2 Mach^2)^(7/2), mu = mu_r (T / T_r)^(3/2)
// (T_r + S) / (T + S), in double as qoi_utils.hpp:135-165 computes them;
// the reference's pow(x, 7) and pow(x, 3) are multiplication chains here.
// Estimates (qoi_utils.hpp:18-98): |V_TOT~ - V_TOT| <= sqrt-rule(V^2,
// sum_f square-rule(V_f, eb_f)) as halving_Vtot.cpp:38-45 forms it, and
// |T~ - T| <= division-rule(P, D, eb_P, eb_D) / R (0 where the rule gives no
// bound, as the reference does). One thread per point, streaming; the
// maxima over the field are reduced with 64-bit atomicMax on the (non-
// negative) doubles' bit patterns.
#include "common.cuh"
#include "kernels.cuh"

namespace prodm {
namespace {

struct Ge {
    static constexpr double R = 287.1, gamma = 1.4, mu_r = 1.716e-5, T_r = 273.15, S = 110.4;
};

// uncontracted, operation by operation as the host evaluates the rules
__device__ __forceinline__ double bx2(double x, double eb) {
    return __dadd_rn(__dmul_rn(__dmul_rn(2.0, fabs(x)), eb), __dmul_rn(eb, eb));
}
__device__ __forceinline__ double bsqrt(double x, double eb) {
    if (x == 0) return sqrt(eb);
    if (x > eb) return eb / __dadd_rn(sqrt(__dsub_rn(x, eb)), sqrt(x));
    return eb / sqrt(x);
}
__device__ __forceinline__ double bdiv(double x, double y, double ebx, double eby) {
    if (eby < fabs(y)) {
        const double e = __dadd_rn(__dmul_rn(fabs(x), eby), __dmul_rn(fabs(y), ebx));
        return y > 0 ? e / __dmul_rn(y, __dsub_rn(y, eby)) : e / __dmul_rn(y, __dadd_rn(y, eby));
    }
    return 0;
}

__global__ void k_qoi_values(const double* __restrict__ vx, const double* __restrict__ vy,
                             const double* __restrict__ vz, const double* __restrict__ p,
                             const double* __restrict__ d, uint64_t n, double* __restrict__ vtot,
                             double* __restrict__ temp, double* __restrict__ cs, double* __restrict__ mach,
                             double* __restrict__ pt, double* __restrict__ mu) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const double v2 = __dadd_rn(__dadd_rn(__dmul_rn(vx[i], vx[i]), __dmul_rn(vy[i], vy[i])), __dmul_rn(vz[i], vz[i]));
        const double v = sqrt(v2);
        const double t = p[i] / __dmul_rn(d[i], Ge::R);
        const double c = sqrt(__dmul_rn(__dmul_rn(Ge::gamma, Ge::R), t));
        const double m = v / c;
        const double mt = __dadd_rn(1.0, __dmul_rn(__dmul_rn((Ge::gamma - 1) / 2, m), m));
        // x^7 and x^3 by multiplication chains instead of pow (GB300's FP64
        // pipe is slow; the chains stay within a few units in the last place)
        const double mt2 = __dmul_rn(mt, mt), mt4 = __dmul_rn(mt2, mt2);
        const double ptv = __dmul_rn(p[i], sqrt(__dmul_rn(__dmul_rn(mt4, mt2), mt)));
        const double trs = (Ge::T_r + Ge::S) / __dadd_rn(t, Ge::S);
        const double tr = t / Ge::T_r;
        const double tt3 = sqrt(__dmul_rn(__dmul_rn(tr, tr), tr));
        vtot[i] = v;
        temp[i] = t;
        cs[i] = c;
        mach[i] = m;
        pt[i] = ptv;
        mu[i] = __dmul_rn(__dmul_rn(Ge::mu_r, tt3), trs);
    }
}

__device__ __forceinline__ void atomic_max_nonneg(double* addr, double v) {
    atomicMax(reinterpret_cast<unsigned long long*>(addr), (unsigned long long)__double_as_longlong(v));
}

__global__ void k_qoi_bounds(const double* __restrict__ vx, const double* __restrict__ vy,
                             const double* __restrict__ vz, const double* __restrict__ p,
                             const double* __restrict__ d, uint64_t n, double ebx, double eby, double ebz, double ebp,
                             double ebd, double* __restrict__ bv, double* __restrict__ bt, double* __restrict__ mx) {
    double mv = 0, mt = 0;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        if (vx) {
            const double e2 = __dadd_rn(__dadd_rn(bx2(vx[i], ebx), bx2(vy[i], eby)), bx2(vz[i], ebz));
            const double v2 =
                __dadd_rn(__dadd_rn(__dmul_rn(vx[i], vx[i]), __dmul_rn(vy[i], vy[i])), __dmul_rn(vz[i], vz[i]));
            const double e = bsqrt(v2, e2);
            if (bv) bv[i] = e;
            mv = e > mv ? e : mv;
        }
        if (p) {
            const double e = __dmul_rn(1.0 / Ge::R, bdiv(p[i], d[i], ebp, ebd));
            if (bt) bt[i] = e;
            mt = e > mt ? e : mt;
        }
    }
    if (mx) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            mv = fmax(mv, __shfl_xor_sync(0xffffffffu, mv, o));
            mt = fmax(mt, __shfl_xor_sync(0xffffffffu, mt, o));
        }
        if ((threadIdx.x & 31) == 0) {
            atomic_max_nonneg(mx, mv);
            atomic_max_nonneg(mx + 1, mt);
        }
    }
}

}  // namespace
}  // namespace prodm

using namespace prodm;

extern "C" {

int prodm_qoi_ge_values(int dtype, const void* vx, const void* vy, const void* vz, const void* p, const void* d,
                        uint64_t n, void* vtot, void* temp, void* c, void* mach, void* pt, void* mu, void* stream) {
    if (dtype != PRODM_F64) return fail(PRODM_EUNSUPPORTED, "prodm_qoi_ge_values: fp64 fields only");
    if (!vx || !vy || !vz || !p || !d || !vtot || !temp || !c || !mach || !pt || !mu)
        return fail(PRODM_EINVAL, "prodm_qoi_ge_values: NULL pointer");
    if (n == 0) return PRODM_OK;
    k_qoi_values<<<grid_for(n, 256), 256, 0, (cudaStream_t)stream>>>(
        (const double*)vx, (const double*)vy, (const double*)vz, (const double*)p, (const double*)d, n,
        (double*)vtot, (double*)temp, (double*)c, (double*)mach, (double*)pt, (double*)mu);
    PRODM_CHECK_LAUNCH("k_qoi_values");
    return PRODM_OK;
}

int prodm_qoi_ge_bounds(int dtype, const void* vx, const void* vy, const void* vz, const void* p, const void* d,
                        uint64_t n, double eb_vx, double eb_vy, double eb_vz, double eb_p, double eb_d,
                        double* bound_vtot, double* bound_t, double* max_bounds, void* stream) {
    if (dtype != PRODM_F64) return fail(PRODM_EUNSUPPORTED, "prodm_qoi_ge_bounds: fp64 fields only");
    const bool v = vx && vy && vz, t = p && d;
    if (!v && !t) return fail(PRODM_EINVAL, "prodm_qoi_ge_bounds: give the velocity fields, or P and D");
    if ((vx || vy || vz) && !v) return fail(PRODM_EINVAL, "prodm_qoi_ge_bounds: all three velocity fields are needed");
    if ((p || d) && !t) return fail(PRODM_EINVAL, "prodm_qoi_ge_bounds: P and D are needed together");
    if (eb_vx < 0 || eb_vy < 0 || eb_vz < 0 || eb_p < 0 || eb_d < 0)
        return fail(PRODM_EINVAL, "prodm_qoi_ge_bounds: error bounds must be non-negative");
    cudaStream_t st = (cudaStream_t)stream;
    if (max_bounds) PRODM_CUDA(cudaMemsetAsync(max_bounds, 0, 2 * sizeof(double), st));
    if (n == 0) return PRODM_OK;
    k_qoi_bounds<<<grid_for(n, 256), 256, 0, st>>>(
        v ? (const double*)vx : nullptr, (const double*)vy, (const double*)vz, t ? (const double*)p : nullptr,
        (const double*)d, n, eb_vx, eb_vy, eb_vz, eb_p, eb_d, bound_vtot, bound_t, max_bounds);
    PRODM_CHECK_LAUNCH("k_qoi_bounds");
    return PRODM_OK;
}

}  // extern "C"
