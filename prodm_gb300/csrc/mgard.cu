// MGARD multilevel decomposition / recomposition kernels (sm_103a).
//
// One level maps the nodal values on a fine box F to
//   * coefficients c(x) = u(x) - (multilinear interpolant of the coarse nodal
//     values)(x) at every non-coarse node, and
//   * the coarse nodal values (orthogonal basis: plus the L2-projection
//     correction z = (M_c^-1 P^T M_f)^{(x)3} c, solved per dim with Thomas).
// Per dim the coarse nodes are the even indices below n-1 plus n-1
// ((n >> 1) + 1 of them, RefactorUtils.hpp:21-34). The reference obtains this
// transform from MGARDx (MGARD.hpp:14-66); MGARDx is not part of the reference
// tree, so the arithmetic here follows the published MGARD method.
//
// Two layouts are supported:
//  * packed   -- level coefficients in interleaved order (the order
//                DirectInterleaver.hpp:23-31 produces) plus a compact coarse
//                box; used by the device-resident pipeline, which never
//                materialises the in-place layout;
//  * in place -- the reference layout: the level box of a strided array,
//                reordered per dim so that coarse nodes come first
//                (DecomposerInterface.hpp:14-16).
#include <cstdlib>

#include "common.cuh"
#include "kernels.cuh"
#include "rows.cuh"

namespace prodm {

namespace {

// Multilinear interpolation at fine node (x0,x1,x2) from its corner values,
// dims averaged with dim 0 outermost (the oracle uses the same order).
template <class T, class Get>
__device__ __forceinline__ T interp(int mask, Get at) {
    auto avg = [&](T a, T b) { return avg_rn(a, b); };
    switch (mask) {
        case 1: return avg(at(-1, 0, 0), at(1, 0, 0));
        case 2: return avg(at(0, -1, 0), at(0, 1, 0));
        case 4: return avg(at(0, 0, -1), at(0, 0, 1));
        case 3: return avg(avg(at(-1, -1, 0), at(-1, 1, 0)), avg(at(1, -1, 0), at(1, 1, 0)));
        case 5: return avg(avg(at(-1, 0, -1), at(-1, 0, 1)), avg(at(1, 0, -1), at(1, 0, 1)));
        case 6: return avg(avg(at(0, -1, -1), at(0, -1, 1)), avg(at(0, 1, -1), at(0, 1, 1)));
        case 7: {
            T a = avg(avg(at(-1, -1, -1), at(-1, -1, 1)), avg(at(-1, 1, -1), at(-1, 1, 1)));
            T b = avg(avg(at(1, -1, -1), at(1, -1, 1)), avg(at(1, 1, -1), at(1, 1, 1)));
            return avg(a, b);
        }
        default: return (T)0;
    }
}

template <class K>
__device__ __forceinline__ K warp_max(K v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        K w = __shfl_xor_sync(0xffffffffu, v, o);
        v = w > v ? w : v;
    }
    return v;
}

// ---------------------------------------------------------------------------
// forward level: in = natural-order fine box (strides s0, s1, 1)
// PACKED:  coef[rank] and coarse[compact C box]
// INPLACE: out[reordered position] with strides o0, o1, 1 (coef and coarse)
// fnat (optional): natural-order coefficient field, zero at coarse nodes
// ---------------------------------------------------------------------------
template <class T, bool PACKED>
__global__ void k_decompose_level(const T* __restrict__ in, uint64_t s0, uint64_t s1, Box F, Box C,
                                  T* __restrict__ coef, T* __restrict__ coarse, uint64_t o0, uint64_t o1,
                                  T* __restrict__ fnat, typename KeyOf<T>::type* maxkey_level,
                                  typename KeyOf<T>::type* maxkey_coarse) {
    using K = typename KeyOf<T>::type;
    K mk = 0, mc = 0;
    const uint64_t total = F.size();
    for (uint64_t idx = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
         idx += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t x2 = (uint32_t)(idx % F.n[2]);
        uint64_t t = idx / F.n[2];
        uint32_t x1 = (uint32_t)(t % F.n[1]);
        uint32_t x0 = (uint32_t)(t / F.n[1]);
        const T* p = in + x0 * s0 + x1 * s1 + x2;
        T v = *p;
        int mask = (is_coarse(x0, F.n[0]) ? 0 : 1) | (is_coarse(x1, F.n[1]) ? 0 : 2) | (is_coarse(x2, F.n[2]) ? 0 : 4);
        uint32_t r0 = reord(x0, F.n[0], C.n[0]), r1 = reord(x1, F.n[1], C.n[1]), r2 = reord(x2, F.n[2], C.n[2]);
        if (mask == 0) {
            if (PACKED) coarse[((uint64_t)r0 * C.n[1] + r1) * C.n[2] + r2] = v;
            else coef[r0 * o0 + r1 * o1 + r2] = v;
            if (fnat) fnat[idx] = (T)0;
            K k = abs_key(v);
            mc = k > mc ? k : mc;
        } else {
            auto at = [&](int d0, int d1, int d2) -> T { return __ldg(p + (int64_t)d0 * (int64_t)s0 + (int64_t)d1 * (int64_t)s1 + d2); };
            T c = sub_rn(v, interp<T>(mask, at));
            if (PACKED) coef[level_rank(r0, r1, r2, F, C)] = c;
            else coef[r0 * o0 + r1 * o1 + r2] = c;
            if (fnat) fnat[idx] = c;
            K k = abs_key(c);
            mk = k > mk ? k : mk;
        }
    }
    if (maxkey_level) {
        mk = warp_max(mk);
        if ((threadIdx.x & 31) == 0 && mk) atomicMax(maxkey_level, mk);
    }
    if (maxkey_coarse) {
        mc = warp_max(mc);
        if ((threadIdx.x & 31) == 0 && mc) atomicMax(maxkey_coarse, mc);
    }
}

// ---------------------------------------------------------------------------
// inverse level: coarse values (already corrected back to nodal values for
// the orthogonal basis) + coefficients -> natural-order fine box.
// PACKED:  coarse = compact C box, coef = packed level coefficients
// INPLACE: both read from a compact reordered copy of the level box (rin)
// ---------------------------------------------------------------------------
template <class T, bool PACKED>
__global__ void k_recompose_level(const T* __restrict__ coarse, const T* __restrict__ coef, Box F, Box C,
                                  T* __restrict__ out, uint64_t s0, uint64_t s1) {
    const uint64_t total = F.size();
    for (uint64_t idx = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
         idx += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t x2 = (uint32_t)(idx % F.n[2]);
        uint64_t t = idx / F.n[2];
        uint32_t x1 = (uint32_t)(t % F.n[1]);
        uint32_t x0 = (uint32_t)(t / F.n[1]);
        int mask = (is_coarse(x0, F.n[0]) ? 0 : 1) | (is_coarse(x1, F.n[1]) ? 0 : 2) | (is_coarse(x2, F.n[2]) ? 0 : 4);
        // coarse-index coordinates of the "low" corner
        uint32_t c0 = (mask & 1) ? (x0 >> 1) : reord(x0, F.n[0], C.n[0]);
        uint32_t c1 = (mask & 2) ? (x1 >> 1) : reord(x1, F.n[1], C.n[1]);
        uint32_t c2 = (mask & 4) ? (x2 >> 1) : reord(x2, F.n[2], C.n[2]);
        T v;
        if (PACKED) {
            const T* cb = coarse + ((uint64_t)c0 * C.n[1] + c1) * C.n[2] + c2;
            const uint64_t cs0 = (uint64_t)C.n[1] * C.n[2], cs1 = C.n[2];
            if (mask == 0) {
                v = *cb;
            } else {
                // corner offsets: -1 -> low corner (0), +1 -> next coarse node (1)
                auto at = [&](int d0, int d1, int d2) -> T {
                    return __ldg(cb + (d0 > 0 ? cs0 : 0) + (d1 > 0 ? cs1 : 0) + (d2 > 0 ? 1 : 0));
                };
                uint32_t r0 = reord(x0, F.n[0], C.n[0]), r1 = reord(x1, F.n[1], C.n[1]), r2 = reord(x2, F.n[2], C.n[2]);
                v = add_rn(coef[level_rank(r0, r1, r2, F, C)], interp<T>(mask, at));
            }
        } else {
            // rin: compact reordered fine box; coarse region = [0,C)
            const uint64_t fs0 = (uint64_t)F.n[1] * F.n[2], fs1 = F.n[2];
            const T* cb = coarse + c0 * fs0 + c1 * fs1 + c2;
            if (mask == 0) {
                v = *cb;
            } else {
                auto at = [&](int d0, int d1, int d2) -> T {
                    return __ldg(cb + (d0 > 0 ? fs0 : 0) + (d1 > 0 ? fs1 : 0) + (d2 > 0 ? 1 : 0));
                };
                uint32_t r0 = reord(x0, F.n[0], C.n[0]), r1 = reord(x1, F.n[1], C.n[1]), r2 = reord(x2, F.n[2], C.n[2]);
                v = add_rn(coef[r0 * fs0 + r1 * fs1 + r2], interp<T>(mask, at));
            }
        }
        out[x0 * s0 + x1 * s1 + x2] = v;
    }
}

// ---------------------------------------------------------------------------
// Row-parallel forms used by the device pipeline (packed layout). One CTA
// walks fine rows (x0, x1); threads stride along x2, so loads and stores are
// coalesced and there is no per-element 64-bit division. Same arithmetic
// (and the same uncontracted operation order) as the generic kernels.
// ---------------------------------------------------------------------------
template <class T>
__global__ void __launch_bounds__(256) k_decompose_rows(const T* __restrict__ in, uint64_t s0, uint64_t s1, Box F, Box C,
                                                        T* __restrict__ coef, T* __restrict__ coarse,
                                                        T* __restrict__ fnat, typename KeyOf<T>::type* maxkey_level,
                                                        typename KeyOf<T>::type* maxkey_coarse) {
    using K = typename KeyOf<T>::type;
    K mk = 0, mc = 0;
    const uint32_t rows = F.n[0] * F.n[1];
    const uint32_t lane = threadIdx.x & 31, wpb = blockDim.x >> 5;
    const bool odd = (F.n[2] & 1u) != 0;
    for (uint32_t row = blockIdx.x * wpb + (threadIdx.x >> 5); row < rows; row += gridDim.x * wpb) {
        if (odd) decompose_row_odd_any<T>(in, s0, s1, F, C, coef, coarse, fnat, row, lane, mk, mc);
        else decompose_row<T>(in, s0, s1, F, C, coef, coarse, fnat, row, lane, mk, mc);
    }
    if (maxkey_level) {
        mk = warp_max_key(mk);
        if ((threadIdx.x & 31) == 0 && mk) atomicMax(maxkey_level, mk);
    }
    if (maxkey_coarse) {
        mc = warp_max_key(mc);
        if ((threadIdx.x & 31) == 0 && mc) atomicMax(maxkey_coarse, mc);
    }
}

// patch form (grids whose every dim is 2 C - 1, no natural-order copy): one
// warp item = coarse columns 32g .. 32g + 31 of a 2 x 2 kPatchSteps strip of
// fine rows (decompose_patch_item)
template <class T>
__global__ void __launch_bounds__(256, sizeof(T) == 4 ? 3 : 2) k_decompose_patch(const T* __restrict__ in, uint64_t s0, uint64_t s1, Box F,
                                                         Box C, T* __restrict__ coef, T* __restrict__ coarse,
                                                         typename KeyOf<T>::type* maxkey_level,
                                                         typename KeyOf<T>::type* maxkey_coarse) {
    using K = typename KeyOf<T>::type;
    K mk = 0, mc = 0;
    const uint64_t items = patch_items(C);
    const uint32_t lane = threadIdx.x & 31, wpb = blockDim.x >> 5;
    for (uint64_t w = (uint64_t)blockIdx.x * wpb + (threadIdx.x >> 5); w < items; w += (uint64_t)gridDim.x * wpb)
        decompose_patch_item<T>(in, s0, s1, F, C, coef, coarse, w, lane, mk, mc);
    if (maxkey_level) {
        mk = warp_max_key(mk);
        if (lane == 0 && mk) atomicMax(maxkey_level, mk);
    }
    if (maxkey_coarse) {
        mc = warp_max_key(mc);
        if (lane == 0 && mc) atomicMax(maxkey_coarse, mc);
    }
}

// patch form of the recomposition (recompose_patch_item), same items as k_decompose_patch
template <class T>
__global__ void __launch_bounds__(256, sizeof(T) == 4 ? 3 : 2) k_recompose_patch(const T* __restrict__ coarse,
                                                                                  const T* __restrict__ coef, Box F,
                                                                                  Box C, T* __restrict__ out,
                                                                                  uint64_t s0, uint64_t s1) {
    pdl_wait();   // the coarse box and the coefficients come from the previous launches
    pdl_release();
    const uint64_t items = patch_items(C);
    const uint32_t lane = threadIdx.x & 31, wpb = blockDim.x >> 5;
    for (uint64_t w = (uint64_t)blockIdx.x * wpb + (threadIdx.x >> 5); w < items; w += (uint64_t)gridDim.x * wpb)
        recompose_patch_item<T>(coarse, coef, F, C, out, s0, s1, w, lane);
}

template <class T>
__global__ void __launch_bounds__(256) k_recompose_rows(const T* __restrict__ coarse, const T* __restrict__ coef, Box F,
                                                        Box C, T* __restrict__ out, uint64_t s0, uint64_t s1) {
    pdl_wait();   // the coarse box and the coefficients come from the previous launches
    pdl_release();
    const uint32_t rows = F.n[0] * F.n[1];
    const uint32_t lane = threadIdx.x & 31, wpb = blockDim.x >> 5;
    const bool odd = (F.n[2] & 1u) != 0;
    for (uint32_t row = blockIdx.x * wpb + (threadIdx.x >> 5); row < rows; row += gridDim.x * wpb) {
        if (odd) recompose_row_odd_any<T>(coarse, coef, F, C, out, s0, s1, row, lane);
        else recompose_row<T>(coarse, coef, F, C, out, s0, s1, row, lane);
    }
}

// copy a box between strided arrays
template <class T>
__global__ void k_copy_box(const T* __restrict__ src, uint64_t a0, uint64_t a1, Box B, T* __restrict__ dst, uint64_t b0,
                           uint64_t b1) {
    const uint64_t total = B.size();
    for (uint64_t idx = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
         idx += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t x2 = (uint32_t)(idx % B.n[2]);
        uint64_t t = idx / B.n[2];
        uint32_t x1 = (uint32_t)(t % B.n[1]);
        uint32_t x0 = (uint32_t)(t / B.n[1]);
        dst[x0 * b0 + x1 * b1 + x2] = src[x0 * a0 + x1 * a1 + x2];
    }
}

// packed coefficients -> natural-order fine field, zeros at coarse nodes
template <class T>
__global__ void k_coef_to_natural(const T* __restrict__ coef, Box F, Box C, T* __restrict__ fnat) {
    const uint64_t total = F.size();
    for (uint64_t idx = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
         idx += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t x2 = (uint32_t)(idx % F.n[2]);
        uint64_t t = idx / F.n[2];
        uint32_t x1 = (uint32_t)(t % F.n[1]);
        uint32_t x0 = (uint32_t)(t / F.n[1]);
        bool c = is_coarse(x0, F.n[0]) && is_coarse(x1, F.n[1]) && is_coarse(x2, F.n[2]);
        T v = (T)0;
        if (!c) {
            uint32_t r0 = reord(x0, F.n[0], C.n[0]), r1 = reord(x1, F.n[1], C.n[1]), r2 = reord(x2, F.n[2], C.n[2]);
            v = coef[level_rank(r0, r1, r2, F, C)];
        }
        fnat[idx] = v;
    }
}

// in-place reordered level box (compact copy) -> natural coefficient field
template <class T>
__global__ void k_reordered_to_natural(const T* __restrict__ rin, Box F, Box C, T* __restrict__ fnat) {
    const uint64_t total = F.size();
    const uint64_t fs0 = (uint64_t)F.n[1] * F.n[2], fs1 = F.n[2];
    for (uint64_t idx = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
         idx += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t x2 = (uint32_t)(idx % F.n[2]);
        uint64_t t = idx / F.n[2];
        uint32_t x1 = (uint32_t)(t % F.n[1]);
        uint32_t x0 = (uint32_t)(t / F.n[1]);
        bool c = is_coarse(x0, F.n[0]) && is_coarse(x1, F.n[1]) && is_coarse(x2, F.n[2]);
        T v = (T)0;
        if (!c) {
            uint32_t r0 = reord(x0, F.n[0], C.n[0]), r1 = reord(x1, F.n[1], C.n[1]), r2 = reord(x2, F.n[2], C.n[2]);
            v = rin[r0 * fs0 + r1 * fs1 + r2];
        }
        fnat[idx] = v;
    }
}

// Right-hand side of the coarse projection at coarse node m of a line of nf
// fine values: b = (M_f s)[c] + 1/2 (M_f s)[c-1] + 1/2 (M_f s)[c+1] with c
// its fine position, the neighbours only when they are not coarse nodes, and
// (M_f s)[x] = dg(x) s[x] + (s[x-1] + s[x+1]) / 6 (P1 mass matrix, dg = 1/3 at
// the ends, else 2/3; s = 0 outside the line). Window: the fine values at
// c-2 .. c+2. For double data an interior node takes the same sum regrouped as
// one 5-point stencil, 5/6 s[c] + 1/2 (s[c-1] + s[c+1]) + 1/12 (s[c-2] + s[c+2]),
// a third of the FP64 operations; float keeps the term order above.
template <class W>
__device__ __forceinline__ W l2_rhs(W sm2, W sm1, W s0, W s1, W s2, uint32_t c, uint32_t nf) {
    if (sizeof(W) == 8 && c >= 2 && c + 3 <= nf && (c & 1u) == 0)
        return (W)(5.0 / 6.0) * s0 + (W)0.5 * (sm1 + s1) + (W)(1.0 / 12.0) * (sm2 + s2);
    auto mf = [&](W l, W x, W r, uint32_t pos) {
        const W dg = (pos == 0 || pos == nf - 1) ? (W)1 / 3 : (W)2 / 3;
        return dg * x + (l + r) / 6;
    };
    W b = mf(sm1, s0, s1, c);
    if (c > 0 && !is_coarse(c - 1, nf)) b += (W)0.5 * mf(sm2, sm1, s0, c - 1);
    if (c + 1 < nf && !is_coarse(c + 1, nf)) b += (W)0.5 * mf(s0, s1, s2, c + 1);
    return b;
}

// One dim of the L2 projection: dst = M_c^-1 P^T M_f src along dim d.
// Thread per line (consecutive threads on consecutive lines of the two
// faster dims, so every access is coalesced across a warp); the fine values
// stream through a 5-value window (two loads per coarse node, issued one
// node ahead), the forward sweep stores d'_m in dst, the backward sweep
// substitutes in place. cp / lo_w / inv_den: Thomas factors of the coarse
// mass matrix (length nc, in W).
template <class T, class W>
__global__ void k_l2_line(const T* __restrict__ src, Box S, int d, T* __restrict__ dst, Box D, const W* __restrict__ cp,
                          const W* __restrict__ lo_w, const W* __restrict__ inv_den) {
    const uint32_t nf = S.n[d], nc = D.n[d];
    const int o1 = d == 0 ? 1 : 0, o2 = d == 2 ? 1 : 2;
    const uint64_t ss[3] = {(uint64_t)S.n[1] * S.n[2], S.n[2], 1};
    const uint64_t ds[3] = {(uint64_t)D.n[1] * D.n[2], D.n[2], 1};
    const uint64_t lines = (uint64_t)S.n[o1] * S.n[o2];
    for (uint64_t li = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; li < lines;
         li += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t q = (uint32_t)(li % S.n[o2]);
        uint32_t p = (uint32_t)(li / S.n[o2]);
        const T* sl = src + p * ss[o1] + q * ss[o2];
        T* dl = dst + p * ds[o1] + q * ds[o2];
        const uint64_t st = ss[d], dt = ds[d];
        if (nf == nc) {
            for (uint32_t x = 0; x < nf; x++) dl[x * dt] = sl[x * st];
            continue;
        }
        auto at = [&](int64_t x) -> W { return (x >= 0 && x < (int64_t)nf) ? (W)sl[x * st] : (W)0; };
        // regular coarse nodes sit at c = 2m; with an even nf the last one is nf - 1
        const uint32_t nreg = (nf & 1u) ? nc : nc - 1;
        W sm2 = 0, sm1 = 0, s0 = at(0), s1 = at(1), s2 = at(2);
        W prev = 0;
        for (uint32_t m = 0; m < nreg; m++) {
            const uint32_t c = 2 * m;
            const W n3 = at((int64_t)c + 3), n4 = at((int64_t)c + 4);   // the next node's new values
            const W b = l2_rhs<W>(sm2, sm1, s0, s1, s2, c, nf);
            const W dp = (m == 0) ? b * inv_den[0] : (b - lo_w[m] * prev) * inv_den[m];
            dl[m * dt] = (T)dp;
            prev = dp;
            sm2 = s0; sm1 = s1; s0 = s2; s1 = n3; s2 = n4;
        }
        if (nreg < nc) {   // even nf: the last coarse node is the last fine node
            const uint32_t c = nf - 1, m = nc - 1;
            const W b = l2_rhs<W>(at((int64_t)c - 2), at((int64_t)c - 1), at(c), (W)0, (W)0, c, nf);
            const W dp = (b - lo_w[m] * prev) * inv_den[m];
            dl[m * dt] = (T)dp;
        }
        W z = (W)dl[(nc - 1) * dt];
        for (uint32_t m = nc - 1; m-- > 0;) {
            z = (W)dl[m * dt] - cp[m] * z;
            dl[m * dt] = (T)z;
        }
    }
}

// The dim-2 (contiguous) pass of the L2 projection with shared-memory staging:
// one warp per 32 lines (fine rows (x0, x1) of F). Forward sweep: tiles of 16
// fine columns plus two halo columns each side are staged with coalesced
// loads (the 32 x 20 values as one flat loop); lane r then sweeps row r's
// coarse nodes of the tile (right-hand side from the 5-point neighbourhood,
// Thomas forward step) into an output tile stored with coalesced writes.
// Backward sweep: the stored values come back from the end in 16-node chunks
// (in the input tile, free by then), lane r substitutes back along its row,
// and they are stored again. About 8 KB of shared memory per warp, so about
// 28 warps share an SM (with 32-column tiles, 14 KB and 15 warps, the
// passes took 9 % longer at 513 x 513 x 257 fp64). PACKED: the rows are read straight from the level's
// packed coefficients (a natural row is an even/odd split of one contiguous
// run of interleaved ranks; coarse nodes of rows inside the coarse box are
// zero), so no natural-order copy is needed; else from a natural field.
constexpr int L2_TILE = 16;                 // fine columns per tile
constexpr int L2_STAGE = L2_TILE + 4;       // staged columns: 2 + 16 + 2
constexpr int L2_IN_LD = L2_STAGE + 1;      // odd stride (no bank conflicts); also holds 16-node chunks
constexpr int L2_OUT_LD = 9;                // up to 9 coarse nodes per tile, odd stride

template <class T, class W, bool PACKED>
__global__ void __launch_bounds__(32) k_l2_rows(const T* __restrict__ src, Box F, Box C, T* __restrict__ dst,
                                                const W* __restrict__ cp, const W* __restrict__ lo_w,
                                                const W* __restrict__ inv_den) {
    __shared__ W sin_[32 * L2_IN_LD];
    __shared__ W sout[32 * L2_OUT_LD];
    const int lane = threadIdx.x;
    const uint32_t nf = F.n[2], nc = coarse_len(nf);
    const uint64_t lines = (uint64_t)F.n[0] * F.n[1];
    const uint32_t c2n = C.n[2];
    const uint64_t l0 = (uint64_t)blockIdx.x * 32;
    if (l0 >= lines) return;
    const int nl = (int)min((uint64_t)32, lines - l0);
    // each row's source (base offset, inside the coarse box or not), computed
    // once by its lane
    __shared__ uint64_t s_base[32];
    __shared__ int s_cc[32];
    if (lane < nl) {
        const uint64_t li = l0 + lane;
        const uint32_t x0 = (uint32_t)(li / F.n[1]), x1 = (uint32_t)(li - (uint64_t)x0 * F.n[1]);
        if (PACKED) {
            const uint32_t r0 = reord(x0, F.n[0], C.n[0]), r1 = reord(x1, F.n[1], C.n[1]);
            const bool cc = r0 < C.n[0] && r1 < C.n[1];
            s_cc[lane] = cc;
            s_base[lane] = level_rank(r0, r1, cc ? c2n : 0u, F, C);
        } else {
            s_cc[lane] = 0;
            s_base[lane] = li * nf;
        }
    }
    __syncwarp();
    auto fine_at = [&](int r, int64_t x) -> W {   // natural column x of row r, 0 outside
        if (x < 0 || x >= (int64_t)nf) return (W)0;
        const uint64_t base = s_base[r];
        if (!PACKED) return (W)src[base + x];
        const uint32_t xx = (uint32_t)x;
        const uint32_t r2 = reord(xx, nf, c2n);
        if (s_cc[r]) return is_coarse(xx, nf) ? (W)0 : (W)src[base + (r2 - c2n)];
        return (W)src[base + r2];
    };
    T* drow = dst + l0 * nc;                       // the warp's rows are consecutive in dst
    if (nc == nf) {   // no coarse subset along this dim: the projection is the identity
        for (int r = 0; r < nl; r++)
            for (uint32_t j = lane; j < nf; j += 32) drow[(uint64_t)r * nc + j] = (T)fine_at(r, j);
        return;
    }
    const uint32_t ntiles = (nf + L2_TILE - 1) / L2_TILE;
    W prev = 0;
    uint32_t m = 0;                                    // next coarse node of the tile
    for (uint32_t t = 0; t < ntiles; t++) {
        const int64_t x0 = (int64_t)t * L2_TILE - 2;   // first staged column
        for (int i = lane; i < nl * L2_STAGE; i += 32) {
            const int r = i / L2_STAGE, j = i - r * L2_STAGE;
            sin_[r * L2_IN_LD + j] = fine_at(r, x0 + j);
        }
        __syncwarp();
        // coarse nodes whose fine position falls in [32t, 32t + 32): the same
        // range for every row
        const uint32_t xe = min((uint32_t)(t + 1) * L2_TILE, nf);
        const uint32_t mt0 = m;
        uint32_t mt1 = mt0;
        while (mt1 < nc && fine_of_coarse(mt1, nf, nc) < xe) mt1++;
        m = mt1;
        if (lane < nl) {
            const W* s = sin_ + lane * L2_IN_LD;
            for (uint32_t mm = mt0; mm < mt1; mm++) {
                const uint32_t c = fine_of_coarse(mm, nf, nc);
                const W* w = s + ((int64_t)c - x0);   // staged columns c-2 .. c+2
                const W b = l2_rhs<W>(w[-2], w[-1], w[0], w[1], w[2], c, nf);
                const W dp = (mm == 0) ? b * inv_den[0] : (b - lo_w[mm] * prev) * inv_den[mm];
                sout[lane * L2_OUT_LD + (mm - mt0)] = dp;
                prev = dp;
            }
        }
        __syncwarp();
        const int cnt = (int)(mt1 - mt0);
        for (int i = lane; i < nl * cnt; i += 32) {
            const int r = i / cnt, j = i - r * cnt;
            drow[(uint64_t)r * nc + mt0 + j] = (T)sout[r * L2_OUT_LD + j];
        }
        __syncwarp();
    }
    // backward substitution, 32-node chunks from the end, in the input tile
    W z = 0;
    uint32_t mhi = nc;
    while (mhi > 0) {
        const uint32_t mlo = mhi > L2_TILE ? mhi - L2_TILE : 0;
        const int cnt = (int)(mhi - mlo);
        for (int i = lane; i < nl * cnt; i += 32) {
            const int r = i / cnt, j = i - r * cnt;
            sin_[r * L2_IN_LD + j] = (W)drow[(uint64_t)r * nc + mlo + j];
        }
        __syncwarp();
        if (lane < nl) {
            W* o = sin_ + lane * L2_IN_LD;
            for (uint32_t mm = mhi; mm-- > mlo;) {
                z = (mm == nc - 1) ? o[mm - mlo] : o[mm - mlo] - cp[mm] * z;
                o[mm - mlo] = z;
            }
        }
        __syncwarp();
        for (int i = lane; i < nl * cnt; i += 32) {
            const int r = i / cnt, j = i - r * cnt;
            drow[(uint64_t)r * nc + mlo + j] = (T)sin_[r * L2_IN_LD + j];
        }
        __syncwarp();
        mhi = mlo;
    }
}

// dst[i] += sign * z[i] over a compact box written into a strided box
template <class T>
__global__ void k_add_box(T* __restrict__ dst, uint64_t b0, uint64_t b1, const T* __restrict__ z, Box B, T sign) {
    const uint64_t total = B.size();
    for (uint64_t idx = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
         idx += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t x2 = (uint32_t)(idx % B.n[2]);
        uint64_t t = idx / B.n[2];
        uint32_t x1 = (uint32_t)(t % B.n[1]);
        uint32_t x0 = (uint32_t)(t / B.n[1]);
        dst[x0 * b0 + x1 * b1 + x2] += sign * z[idx];
    }
}

// DirectInterleaver gather/scatter over box(fine) \ box(coarse).
template <class T, bool GATHER>
__global__ void k_interleave(T* __restrict__ data, uint64_t s0, uint64_t s1, Box F, Box C, T* __restrict__ buf) {
    const uint64_t total = F.size();
    for (uint64_t idx = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
         idx += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t x2 = (uint32_t)(idx % F.n[2]);
        uint64_t t = idx / F.n[2];
        uint32_t x1 = (uint32_t)(t % F.n[1]);
        uint32_t x0 = (uint32_t)(t / F.n[1]);
        if (x0 < C.n[0] && x1 < C.n[1] && x2 < C.n[2]) continue;
        uint64_t r = level_rank(x0, x1, x2, F, C);
        if (GATHER) buf[r] = data[x0 * s0 + x1 * s1 + x2];
        else data[x0 * s0 + x1 * s1 + x2] = buf[r];
    }
}

}  // namespace

// ---------------------------------------------------------------------------
// host launchers
// ---------------------------------------------------------------------------
// one warp per row, 8 warps per CTA; enough CTAs for full occupancy
unsigned row_threads(uint32_t) { return 256; }
// PRODM_DECOMPOSE_PATCH=0 keeps every level on the row kernels (decomposition and
// recomposition; read per launch)
bool decompose_patch_enabled() {
    const char* v = getenv("PRODM_DECOMPOSE_PATCH");
    return !(v && v[0] == '0');
}
unsigned row_grid(uint64_t rows, unsigned th) {
    const uint64_t wpb = th / 32;
    uint64_t need = (rows + wpb - 1) / wpb;
    uint64_t cap = (uint64_t)device_sms() * 8 * 4;
    uint64_t g = need < cap ? need : cap;
    return (unsigned)(g ? g : 1);
}

template <class T>
int launch_decompose_level_packed(const T* in, uint64_t s0, uint64_t s1, const Box& F, const Box& C, T* coef, T* coarse,
                                  T* fnat, void* maxkey_level, void* maxkey_coarse, cudaStream_t st) {
    using K = typename KeyOf<T>::type;
    const unsigned th = row_threads(F.n[2]);
    if (!fnat && patch_level(F, C) && decompose_patch_enabled()) {
        k_decompose_patch<T><<<row_grid(patch_items(C), th), th, 0, st>>>(in, s0, s1, F, C, coef, coarse,
                                                                          (K*)maxkey_level, (K*)maxkey_coarse);
        PRODM_CHECK_LAUNCH("k_decompose_patch");
        return PRODM_OK;
    }
    k_decompose_rows<T><<<row_grid((uint64_t)F.n[0] * F.n[1], th), th, 0, st>>>(in, s0, s1, F, C, coef, coarse, fnat,
                                                                                 (K*)maxkey_level, (K*)maxkey_coarse);
    PRODM_CHECK_LAUNCH("k_decompose_rows");
    return PRODM_OK;
}

template <class T>
int launch_decompose_level_inplace(const T* in, const Box& F, const Box& C, T* out, uint64_t o0, uint64_t o1, T* fnat,
                                   cudaStream_t st) {
    const int th = 256;
    k_decompose_level<T, false><<<grid_for(F.size(), th), th, 0, st>>>(
        in, (uint64_t)F.n[1] * F.n[2], F.n[2], F, C, out, nullptr, o0, o1, fnat, nullptr, nullptr);
    PRODM_CHECK_LAUNCH("k_decompose_level");
    return PRODM_OK;
}

template <class T>
int launch_recompose_level_packed(const T* coarse, const T* coef, const Box& F, const Box& C, T* out, uint64_t s0,
                                  uint64_t s1, cudaStream_t st, bool pdl) {
    const unsigned th = row_threads(F.n[2]);
    count_launch();
    if (patch_level(F, C) && decompose_patch_enabled()) {
        const cudaError_t e = launch_chain(pdl, k_recompose_patch<T>, dim3(row_grid(patch_items(C), th)), dim3(th), 0,
                                           st, coarse, coef, F, C, out, s0, s1);
        if (e != cudaSuccess) return cuda_status(e, "k_recompose_patch");
        return PRODM_OK;
    }
    const cudaError_t e = launch_chain(pdl, k_recompose_rows<T>, dim3(row_grid((uint64_t)F.n[0] * F.n[1], th)), dim3(th),
                                       0, st, coarse, coef, F, C, out, s0, s1);
    if (e != cudaSuccess) return cuda_status(e, "k_recompose_rows");
    return PRODM_OK;
}

template <class T>
int launch_recompose_level_inplace(const T* rin, const Box& F, const Box& C, T* out, uint64_t s0, uint64_t s1,
                                   cudaStream_t st) {
    const int th = 256;
    k_recompose_level<T, false><<<grid_for(F.size(), th), th, 0, st>>>(rin, rin, F, C, out, s0, s1);
    PRODM_CHECK_LAUNCH("k_recompose_level");
    return PRODM_OK;
}

template <class T>
int launch_copy_box(const T* src, uint64_t a0, uint64_t a1, const Box& B, T* dst, uint64_t b0, uint64_t b1,
                    cudaStream_t st) {
    const int th = 256;
    k_copy_box<T><<<grid_for(B.size(), th), th, 0, st>>>(src, a0, a1, B, dst, b0, b1);
    PRODM_CHECK_LAUNCH("k_copy_box");
    return PRODM_OK;
}

template <class T>
int launch_coef_to_natural(const T* coef, const Box& F, const Box& C, T* fnat, cudaStream_t st) {
    const int th = 256;
    k_coef_to_natural<T><<<grid_for(F.size(), th), th, 0, st>>>(coef, F, C, fnat);
    PRODM_CHECK_LAUNCH("k_coef_to_natural");
    return PRODM_OK;
}

template <class T>
int launch_reordered_to_natural(const T* rin, const Box& F, const Box& C, T* fnat, cudaStream_t st) {
    const int th = 256;
    k_reordered_to_natural<T><<<grid_for(F.size(), th), th, 0, st>>>(rin, F, C, fnat);
    PRODM_CHECK_LAUNCH("k_reordered_to_natural");
    return PRODM_OK;
}

// Thomas factors of the coarse mass matrix of a dim with n fine nodes.
// layout in tab: [cp(nc) | lo(nc) | inv_den(nc)]
template <class W>
void mass_factors(uint32_t n, W* tab) {
    uint32_t nc = coarse_len(n);
    W* cp = tab;
    W* lo = tab + nc;
    W* inv = tab + 2 * nc;
    double prev_cp = 0;
    for (uint32_t m = 0; m < nc; m++) {
        double hl = m > 0 ? (double)(fine_of_coarse(m, n, nc) - fine_of_coarse(m - 1, n, nc)) : 0.0;
        double hr = m + 1 < nc ? (double)(fine_of_coarse(m + 1, n, nc) - fine_of_coarse(m, n, nc)) : 0.0;
        double dg = (hl + hr) / 3, up = hr / 6, low = hl / 6;
        double den = m == 0 ? dg : dg - low * prev_cp;
        double c = up / den;
        cp[m] = (W)c;
        lo[m] = (W)low;
        inv[m] = (W)(1.0 / den);
        prev_cp = c;
    }
}
template void mass_factors<float>(uint32_t, float*);
template void mass_factors<double>(uint32_t, double*);

// z (compact C box) = L2 projection of the natural coefficient field (F box):
// from fnat, or (coef != nullptr) straight from the level's packed
// coefficients (coarse box C). tabs[d] = device Thomas factors for dim d;
// t1/t2 scratch boxes. The contiguous dim goes first through the staged row
// kernel, the two strided dims through the line kernel (coalesced there).
template <class T>
int launch_l2_correction(const T* fnat, const Box& F, T* t1, T* t2, T* z, const T* const tabs[3], cudaStream_t st,
                         const T* coef, const Box* C) {
    const int th = 128;
    Box a = F;
    T* bufs[3] = {t1, t2, z};
    {
        const uint32_t nc = coarse_len(F.n[2]);
        const T* tab = tabs[2];
        const uint64_t lines = (uint64_t)F.n[0] * F.n[1];
        const unsigned grid = (unsigned)((lines + 31) / 32);
        if (coef) k_l2_rows<T, T, true><<<grid, 32, 0, st>>>(coef, F, *C, t1, tab, tab + nc, tab + 2 * nc);
        else k_l2_rows<T, T, false><<<grid, 32, 0, st>>>(fnat, F, F, t1, tab, tab + nc, tab + 2 * nc);
        PRODM_CHECK_LAUNCH("k_l2_rows");
        a.n[2] = nc;
    }
    const T* src = t1;
    for (int k = 1, d = 1; d >= 0; d--, k++) {
        Box b = a;
        b.n[d] = coarse_len(a.n[d]);
        uint64_t lines = a.size() / a.n[d];
        uint32_t nc = b.n[d];
        const T* tab = tabs[d];
        k_l2_line<T, T><<<grid_for(lines, th, 16), th, 0, st>>>(src, a, d, bufs[k], b, tab, tab + nc, tab + 2 * nc);
        PRODM_CHECK_LAUNCH("k_l2_line");
        src = bufs[k];
        a = b;
    }
    return PRODM_OK;
}

template <class T>
int launch_add_box(T* dst, uint64_t b0, uint64_t b1, const T* z, const Box& B, T sign, cudaStream_t st) {
    const int th = 256;
    k_add_box<T><<<grid_for(B.size(), th), th, 0, st>>>(dst, b0, b1, z, B, sign);
    PRODM_CHECK_LAUNCH("k_add_box");
    return PRODM_OK;
}

template <class T>
int launch_interleave(T* data, uint64_t s0, uint64_t s1, const Box& F, const Box& C, T* buf, bool gather,
                      cudaStream_t st) {
    const int th = 256;
    if (gather) k_interleave<T, true><<<grid_for(F.size(), th), th, 0, st>>>(data, s0, s1, F, C, buf);
    else k_interleave<T, false><<<grid_for(F.size(), th), th, 0, st>>>(data, s0, s1, F, C, buf);
    PRODM_CHECK_LAUNCH("k_interleave");
    return PRODM_OK;
}

#define INST(T)                                                                                                     \
    template int launch_decompose_level_packed<T>(const T*, uint64_t, uint64_t, const Box&, const Box&, T*, T*, T*, \
                                                  void*, void*, cudaStream_t);                                      \
    template int launch_decompose_level_inplace<T>(const T*, const Box&, const Box&, T*, uint64_t, uint64_t, T*,    \
                                                   cudaStream_t);                                                   \
    template int launch_recompose_level_packed<T>(const T*, const T*, const Box&, const Box&, T*, uint64_t,         \
                                                  uint64_t, cudaStream_t, bool);                                    \
    template int launch_recompose_level_inplace<T>(const T*, const Box&, const Box&, T*, uint64_t, uint64_t,        \
                                                   cudaStream_t);                                                   \
    template int launch_copy_box<T>(const T*, uint64_t, uint64_t, const Box&, T*, uint64_t, uint64_t, cudaStream_t); \
    template int launch_coef_to_natural<T>(const T*, const Box&, const Box&, T*, cudaStream_t);                     \
    template int launch_reordered_to_natural<T>(const T*, const Box&, const Box&, T*, cudaStream_t);                \
    template int launch_l2_correction<T>(const T*, const Box&, T*, T*, T*, const T* const[3], cudaStream_t,      \
                                         const T*, const Box*);                                                     \
    template int launch_add_box<T>(T*, uint64_t, uint64_t, const T*, const Box&, T, cudaStream_t);                  \
    template int launch_interleave<T>(T*, uint64_t, uint64_t, const Box&, const Box&, T*, bool, cudaStream_t);
INST(float)
INST(double)
#undef INST

}  // namespace prodm
