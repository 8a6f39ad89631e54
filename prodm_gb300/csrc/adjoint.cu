// Adjoint of the hierarchical recomposition (sm_103a).
//
// The retrieval's recomposition is a linear map R from the packed level
// coefficients (level 0 box, then box(l) \ box(l-1) of every level in
// interleaved order, the layout of the device coefficient buffer) to the
// natural-order field. One level is
//   V(x) = C(c)                     at the coarse node x = fine(c)
//   V(x) = coef(x) + sum_corners w C at every other node (w = 2^-#odd dims)
// so its transpose, applied to a field gradient G, is
//   g_coef(x) = G(x)                                    (a gather by rank)
//   g_C(c)    = sum_{d in {-1,0,1}^3} 2^-|d| G(fine(c) + d)
// where each nonzero offset must land on an odd (non-coarse) node, whose
// interpolation then has fine(c) as one of its corners. Each output is
// written by exactly one thread, in a fixed summation order, so the result
// is deterministic. Levels run fine -> coarse through two ping-pong boxes.
#include "common.cuh"
#include "kernels.cuh"

namespace prodm {

namespace {

// gradient of the level-l coefficients: one thread per fine node
template <class T>
__global__ void k_adj_coef(const T* __restrict__ g, Box F, Box C, T* __restrict__ gcoef) {
    const uint64_t N = F.size();
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < N; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t x2 = (uint32_t)(i % F.n[2]);
        const uint64_t r = i / F.n[2];
        const uint32_t x1 = (uint32_t)(r % F.n[1]), x0 = (uint32_t)(r / F.n[1]);
        const bool c0 = is_coarse(x0, F.n[0]), c1 = is_coarse(x1, F.n[1]), c2 = is_coarse(x2, F.n[2]);
        if (c0 && c1 && c2) continue;
        const uint64_t rank = level_rank(reord(x0, F.n[0], C.n[0]), reord(x1, F.n[1], C.n[1]),
                                         reord(x2, F.n[2], C.n[2]), F, C);
        gcoef[rank] = g[i];
    }
}

// offsets along one dim that reach odd nodes having X as a corner
__device__ __forceinline__ int odd_neighbours(uint32_t X, uint32_t n, int (&off)[3]) {
    int k = 0;
    off[k++] = 0;
    if (X >= 1 && !is_coarse(X - 1, n)) off[k++] = -1;
    if (X + 1 < n && !is_coarse(X + 1, n)) off[k++] = 1;
    return k;
}

// gradient of the coarse box: one thread per coarse node
template <class T>
__global__ void k_adj_coarse(const T* __restrict__ g, Box F, Box C, T* __restrict__ gc) {
    const uint64_t N = C.size();
    const uint64_t s0 = (uint64_t)F.n[1] * F.n[2], s1 = F.n[2];
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < N; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t c2 = (uint32_t)(i % C.n[2]);
        const uint64_t r = i / C.n[2];
        const uint32_t c1 = (uint32_t)(r % C.n[1]), c0 = (uint32_t)(r / C.n[1]);
        const uint32_t X0 = fine_of_coarse(c0, F.n[0], C.n[0]);
        const uint32_t X1 = fine_of_coarse(c1, F.n[1], C.n[1]);
        const uint32_t X2 = fine_of_coarse(c2, F.n[2], C.n[2]);
        int o0[3], o1[3], o2[3];
        const int k0 = odd_neighbours(X0, F.n[0], o0);
        const int k1 = odd_neighbours(X1, F.n[1], o1);
        const int k2 = odd_neighbours(X2, F.n[2], o2);
        T acc = 0;
        for (int a = 0; a < k0; a++)
            for (int b = 0; b < k1; b++)
                for (int c = 0; c < k2; c++) {
                    const int odd = (o0[a] != 0) + (o1[b] != 0) + (o2[c] != 0);
                    const T w = odd == 0 ? (T)1 : odd == 1 ? (T)0.5 : odd == 2 ? (T)0.25 : (T)0.125;
                    const uint64_t idx = (uint64_t)(X0 + o0[a]) * s0 + (uint64_t)(X1 + o1[b]) * s1 + (X2 + o2[c]);
                    acc += w * g[idx];
                }
        gc[i] = acc;
    }
}

// ---------------------------------------------------------------------------
// Orthogonal basis. Its recomposition of one level first removes the L2
// correction from the coarse box, C' = C - Q f (f: the level's coefficients on
// the fine box, zero at the coarse-box nodes; Q = Q0 Q1 Q2, one line operator
// per dim, Qd = Mc^-1 R Mf: fine P1 mass matrix, restriction with weights 1
// and 1/2, coarse mass-matrix solve), then interpolates as the hierarchical
// basis. So its transpose takes g_C = g_C' and g_f = g_f(hier) - Q^T g_C',
// Q^T = Q2^T Q1^T Q0^T with Qd^T = Mf R^T Mc^-1 (both mass matrices are
// symmetric): per dim, a tridiagonal solve on the coarse lines, then the
// interpolation (R^T) and the fine mass matrix on the fine lines.
// ---------------------------------------------------------------------------

// the lines of a box along dim d: line li -> (p, q) over the two other dims,
// consecutive li on the faster one (coalesced across a warp)
__device__ __forceinline__ void line_origin(const Box& S, int d, uint64_t li, uint64_t& off_s, const Box& D,
                                            uint64_t& off_d) {
    const int o1 = d == 0 ? 1 : 0, o2 = d == 2 ? 1 : 2;
    const uint64_t ss[3] = {(uint64_t)S.n[1] * S.n[2], S.n[2], 1};
    const uint64_t ds[3] = {(uint64_t)D.n[1] * D.n[2], D.n[2], 1};
    const uint32_t q = (uint32_t)(li % S.n[o2]);
    const uint32_t p = (uint32_t)(li / S.n[o2]);
    off_s = p * ss[o1] + q * ss[o2];
    off_d = p * ds[o1] + q * ds[o2];
}

// u = Mc^-1 y along dim d of box S (coarse length S.n[d]); Thomas factors
// cp / lo_w / inv_den as the forward correction's; u may be y (in place)
template <class T>
__global__ void k_adj_solve(const T* y, Box S, int d, T* u, const T* __restrict__ cp,
                            const T* __restrict__ lo_w, const T* __restrict__ inv_den) {
    const uint32_t nc = S.n[d];
    const uint64_t st = d == 0 ? (uint64_t)S.n[1] * S.n[2] : d == 1 ? S.n[2] : 1;
    const uint64_t lines = S.size() / nc;
    for (uint64_t li = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; li < lines;
         li += (uint64_t)gridDim.x * blockDim.x) {
        uint64_t os, od;
        line_origin(S, d, li, os, S, od);
        const T* yl = y + os;
        T* ul = u + os;
        T prev = 0;
        for (uint32_t m = 0; m < nc; m++) {
            const T b = yl[m * st];
            const T dp = (m == 0) ? b * inv_den[0] : (b - lo_w[m] * prev) * inv_den[m];
            ul[m * st] = dp;
            prev = dp;
        }
        T z = ul[(uint64_t)(nc - 1) * st];
        for (uint32_t m = nc - 1; m-- > 0;) {
            z = ul[m * st] - cp[m] * z;
            ul[m * st] = z;
        }
    }
}

// w = Mf R^T u along dim d: u on box S (coarse length nc along d), w on box D
// (fine length nf). v = R^T u is u at the coarse nodes and the mean of the two
// coarse neighbours at the others; w(x) = dg(x) v(x) + (v(x-1) + v(x+1)) / 6
// (dg = 1/3 at the ends, else 2/3; v = 0 outside). One pass with a window.
template <class T>
__global__ void k_adj_spread(const T* __restrict__ u, Box S, int d, T* __restrict__ w, Box D) {
    const uint32_t nc = S.n[d], nf = D.n[d];
    const uint64_t ss = d == 0 ? (uint64_t)S.n[1] * S.n[2] : d == 1 ? S.n[2] : 1;
    const uint64_t ds = d == 0 ? (uint64_t)D.n[1] * D.n[2] : d == 1 ? D.n[2] : 1;
    const uint64_t lines = S.size() / nc;
    for (uint64_t li = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; li < lines;
         li += (uint64_t)gridDim.x * blockDim.x) {
        uint64_t os, od;
        line_origin(S, d, li, os, D, od);
        const T* ul = u + os;
        T* wl = w + od;
        if (nc == nf) {   // no coarse subset along this dim: the operator is the identity
            for (uint32_t x = 0; x < nf; x++) wl[x * ds] = ul[x * ss];
            continue;
        }
        auto v_at = [&](uint32_t x) -> T {   // R^T u at fine node x (0 <= x < nf)
            if (is_coarse(x, nf)) return ul[(uint64_t)reord(x, nf, nc) * ss];
            return (T)0.5 * ul[(uint64_t)reord(x - 1, nf, nc) * ss] + (T)0.5 * ul[(uint64_t)reord(x + 1, nf, nc) * ss];
        };
        T vl = 0, vx = v_at(0);
        for (uint32_t x = 0; x < nf; x++) {
            const T vr = x + 1 < nf ? v_at(x + 1) : (T)0;
            const T dg = (x == 0 || x == nf - 1) ? (T)1 / 3 : (T)2 / 3;
            wl[x * ds] = dg * vx + (vl + vr) / 6;
            vl = vx;
            vx = vr;
        }
    }
}

// gradient of the level-l coefficients with the correction's share removed:
// gcoef(rank(x)) = G(x) - W(x) at every fine node outside the coarse box
template <class T>
__global__ void k_adj_coef_minus(const T* __restrict__ g, const T* __restrict__ wv, Box F, Box C,
                                 T* __restrict__ gcoef) {
    const uint64_t N = F.size();
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < N; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t x2 = (uint32_t)(i % F.n[2]);
        const uint64_t r = i / F.n[2];
        const uint32_t x1 = (uint32_t)(r % F.n[1]), x0 = (uint32_t)(r / F.n[1]);
        const bool c0 = is_coarse(x0, F.n[0]), c1 = is_coarse(x1, F.n[1]), c2 = is_coarse(x2, F.n[2]);
        if (c0 && c1 && c2) continue;
        const uint64_t rank = level_rank(reord(x0, F.n[0], C.n[0]), reord(x1, F.n[1], C.n[1]),
                                         reord(x2, F.n[2], C.n[2]), F, C);
        gcoef[rank] = g[i] - wv[i];
    }
}

}  // namespace

// transpose of one orthogonal recomposition level: g (box F) -> gcoef (packed
// level coefficients) and gcoarse (box C). tabs[d]: Thomas factors of dim d;
// scratch: boxes (n0, c1, c2), (n0, n1, c2), F and one C box.
template <class T>
int launch_recompose_adjoint_level_orth(const T* g, const Box& F, const Box& C, T* gcoef, T* gcoarse,
                                        const T* const tabs[3], T* s_a, T* s_b, T* s_w, T* s_u, cudaStream_t st) {
    const int th = 256;
    k_adj_coarse<T><<<grid_for(C.size(), th), th, 0, st>>>(g, F, C, gcoarse);
    PRODM_CHECK_LAUNCH("k_adj_coarse");
    // Q0^T, Q1^T, Q2^T: C -> (n0, c1, c2) -> (n0, n1, c2) -> F
    Box a = C;
    const T* src = gcoarse;
    T* outs[3] = {s_a, s_b, s_w};
    for (int d = 0; d < 3; d++) {
        Box b = a;
        b.n[d] = F.n[d];
        const uint32_t nc = a.n[d];
        const uint64_t lines = a.size() / nc;
        if (nc != F.n[d]) {   // in place on the previous scratch box; gcoarse itself stays (it is g_C)
            const T* tab = tabs[d];
            T* u = d == 0 ? s_u : const_cast<T*>(src);
            k_adj_solve<T><<<grid_for(lines, th, 16), th, 0, st>>>(src, a, d, u, tab, tab + nc, tab + 2 * nc);
            PRODM_CHECK_LAUNCH("k_adj_solve");
            src = u;
        }
        k_adj_spread<T><<<grid_for(lines, th, 16), th, 0, st>>>(src, a, d, outs[d], b);
        PRODM_CHECK_LAUNCH("k_adj_spread");
        src = outs[d];
        a = b;
    }
    k_adj_coef_minus<T><<<grid_for(F.size(), th), th, 0, st>>>(g, s_w, F, C, gcoef);
    PRODM_CHECK_LAUNCH("k_adj_coef_minus");
    return PRODM_OK;
}

template int launch_recompose_adjoint_level_orth<float>(const float*, const Box&, const Box&, float*, float*,
                                                        const float* const[3], float*, float*, float*, float*,
                                                        cudaStream_t);
template int launch_recompose_adjoint_level_orth<double>(const double*, const Box&, const Box&, double*, double*,
                                                         const double* const[3], double*, double*, double*, double*,
                                                         cudaStream_t);

template <class T>
int launch_recompose_adjoint_level(const T* g, const Box& F, const Box& C, T* gcoef, T* gcoarse, cudaStream_t st) {
    const int th = 256;
    k_adj_coef<T><<<grid_for(F.size(), th), th, 0, st>>>(g, F, C, gcoef);
    PRODM_CHECK_LAUNCH("k_adj_coef");
    k_adj_coarse<T><<<grid_for(C.size(), th), th, 0, st>>>(g, F, C, gcoarse);
    PRODM_CHECK_LAUNCH("k_adj_coarse");
    return PRODM_OK;
}

template int launch_recompose_adjoint_level<float>(const float*, const Box&, const Box&, float*, float*, cudaStream_t);
template int launch_recompose_adjoint_level<double>(const double*, const Box&, const Box&, double*, double*,
                                                    cudaStream_t);

}  // namespace prodm
