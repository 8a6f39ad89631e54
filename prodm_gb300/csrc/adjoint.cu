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

}  // namespace

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
