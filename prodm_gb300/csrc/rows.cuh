// Per-row bodies of the row-parallel MGARD kernels (one warp per fine row),
// shared by the single-field kernels and the multi-field batched kernels.
#pragma once
#include "common.cuh"

namespace prodm {

template <class K>
__device__ __forceinline__ K warp_max_key(K v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        K w = __shfl_xor_sync(0xffffffffu, v, o);
        v = w > v ? w : v;
    }
    return v;
}

__device__ __forceinline__ uint64_t row_rank_base(uint32_t r0, uint32_t r1, const Box& F, const Box& C, bool& cc) {
    cc = r0 < C.n[0] && r1 < C.n[1];
    // rank of (r0, r1, cc ? C2 : 0)
    return level_rank(r0, r1, cc ? C.n[2] : 0u, F, C);
}

// corner row offsets (elements) of a row for mask m01, in corner_tree order
__device__ __forceinline__ void corner_offsets(int m01, int64_t lo0, int64_t hi0, int64_t lo1, int64_t hi1,
                                               int64_t* o) {
    if (m01 == 0) { o[0] = 0; }
    else if (m01 == 1) { o[0] = lo0; o[1] = hi0; }
    else if (m01 == 2) { o[0] = lo1; o[1] = hi1; }
    else { o[0] = lo0 + lo1; o[1] = lo0 + hi1; o[2] = hi0 + lo1; o[3] = hi0 + hi1; }
}

// forward level on fine row `row` (natural order, strides s0, s1, 1):
// coefficients to coef (interleaved ranks), coarse nodes to coarse (compact C
// box), optional natural coefficient field fnat; running |max| keys in mk / mc
template <class T>
__device__ __forceinline__ void decompose_row(const T* __restrict__ in, uint64_t s0, uint64_t s1, const Box& F,
                                              const Box& C, T* __restrict__ coef, T* __restrict__ coarse,
                                              T* __restrict__ fnat, uint32_t row, uint32_t lane,
                                              typename KeyOf<T>::type& mk, typename KeyOf<T>::type& mc) {
    using K = typename KeyOf<T>::type;
    const uint32_t n2 = F.n[2], c2n = C.n[2];
    const uint32_t x0 = row / F.n[1], x1 = row - x0 * F.n[1];
    const int m01 = (is_coarse(x0, F.n[0]) ? 0 : 1) | (is_coarse(x1, F.n[1]) ? 0 : 2);
    const uint32_t r0 = reord(x0, F.n[0], C.n[0]), r1 = reord(x1, F.n[1], C.n[1]);
    bool cc;
    const uint64_t rbase = row_rank_base(r0, r1, F, C, cc);
    const T* p = in + x0 * s0 + x1 * s1;
    int64_t co[4];
    corner_offsets(m01, -(int64_t)s0, (int64_t)s0, -(int64_t)s1, (int64_t)s1, co);
    const int nq = corner_count(m01);
    T* frow = fnat ? fnat + (uint64_t)row * n2 : nullptr;
    T* crow = coarse + ((uint64_t)r0 * C.n[1] + r1) * c2n;
#pragma unroll 3
    for (uint32_t cbase = 0; cbase < c2n; cbase += 32) {
        const uint32_t c2 = cbase + lane;
        const bool act = c2 < c2n;
        const uint32_t xe = act ? fine_of_coarse(c2, n2, c2n) : 0;
        const bool odd = act && c2 + 1 < c2n && fine_of_coarse(c2 + 1, n2, c2n) == 2 * c2 + 2;
        T q[4] = {0, 0, 0, 0}, qn[4];
        const T ve = act ? p[xe] : (T)0;
        if (m01 == 0) q[0] = ve;
        else {
#pragma unroll
            for (int i = 0; i < 4; i++)
                if (i < nq && act) q[i] = __ldg(p + xe + co[i]);
        }
#pragma unroll
        for (int i = 0; i < 4; i++) {
            qn[i] = __shfl_down_sync(0xffffffffu, q[i], 1);
            if (i < nq && lane == 31 && odd) {
                const uint32_t xn = 2 * c2 + 2;
                qn[i] = m01 == 0 ? p[xn] : __ldg(p + xn + co[i]);
            }
        }
        if (act) {
            if (m01 == 0) {
                crow[c2] = ve;
                if (frow) frow[xe] = (T)0;
                K k = abs_key(ve);
                mc = k > mc ? k : mc;
            } else {
                T c = sub_rn(ve, corner_tree(m01, q));
                coef[rbase + (cc ? c2 - c2n : c2)] = c;
                if (frow) frow[xe] = c;
                K k = abs_key(c);
                mk = k > mk ? k : mk;
            }
            if (odd) {
                const uint32_t xo = 2 * c2 + 1;
                T c = sub_rn(p[xo], corner_tree_mid(m01, q, qn));
                coef[rbase + (cc ? c2 : c2n + c2)] = c;
                if (frow) frow[xo] = c;
                K k = abs_key(c);
                mk = k > mk ? k : mk;
            }
        }
    }
}

// ---------------------------------------------------------------------------
// Odd row length (fine node 2c = coarse node c, odd node 2c+1 between coarse
// nodes c and c+1; n = 2^k + 1 and every other odd n). Lane l handles coarse
// columns 32k + l; the loads of D column groups are in flight at once in a
// register ring refilled as each group is used, so a row waits for the memory
// latency about once rather than once per group. The next column's corner
// values come from lane l+1 by shuffle, and lane 31 takes lane 0 of the next
// group from the ring. Same arithmetic as decompose_row / recompose_row.
// ---------------------------------------------------------------------------
template <class T, int M01>
__device__ __forceinline__ void decompose_row_odd(const T* __restrict__ p, uint64_t s0, uint64_t s1, uint32_t c2n,
                                                  T* __restrict__ coef, uint64_t rb_even, uint64_t rb_odd,
                                                  T* __restrict__ crow, T* __restrict__ frow, uint32_t lane,
                                                  typename KeyOf<T>::type& mk, typename KeyOf<T>::type& mc) {
    using K = typename KeyOf<T>::type;
    constexpr int NQ = M01 == 0 ? 1 : (M01 == 3 ? 4 : 2);
    constexpr int D = M01 == 3 ? 4 : 6;   // ring depth (measured at 513^3: 3/4 -> 256 us, 4/6 -> 241 us, 5/8 -> 250 us)
    int64_t co[4];
    corner_offsets(M01, -(int64_t)s0, (int64_t)s0, -(int64_t)s1, (int64_t)s1, co);
    struct G { T ve, vo, q[NQ]; };
    auto load = [&](uint32_t k, G& g) {
        const uint32_t c = 32 * k + lane;
        const bool a = c < c2n, o = c + 1 < c2n;
        const T* e = p + 2 * (uint64_t)c;
        g.ve = a ? e[0] : (T)0;
        g.vo = o ? e[1] : (T)0;
        if (M01 == 0) g.q[0] = g.ve;
        else {
#pragma unroll
            for (int i = 0; i < NQ; i++) g.q[i] = a ? __ldg(e + co[i]) : (T)0;
        }
    };
    const uint32_t groups = (c2n + 31) / 32;
    G ring[D];
#pragma unroll
    for (int d = 0; d < D; d++) load(d, ring[d]);
    for (uint32_t k0 = 0; k0 < groups; k0 += D) {
#pragma unroll
        for (int d = 0; d < D; d++) {
            const uint32_t k = k0 + d;
            if (k >= groups) break;
            const G& g = ring[d];
            const G& gx = ring[(d + 1) % D];
            T qn[NQ];
#pragma unroll
            for (int i = 0; i < NQ; i++) qn[i] = __shfl_sync(0xffffffffu, lane == 0 ? gx.q[i] : g.q[i], (lane + 1) & 31);
            const uint32_t c2 = 32 * k + lane;
            if (c2 < c2n) {
                if (M01 == 0) {
                    crow[c2] = g.ve;
                    if (frow) frow[2 * (uint64_t)c2] = (T)0;
                    K kk = abs_key(g.ve);
                    mc = kk > mc ? kk : mc;
                } else {
                    T c = sub_rn(g.ve, corner_tree(M01, g.q));
                    coef[rb_even + c2] = c;
                    if (frow) frow[2 * (uint64_t)c2] = c;
                    K kk = abs_key(c);
                    mk = kk > mk ? kk : mk;
                }
                if (c2 + 1 < c2n) {
                    T c = sub_rn(g.vo, corner_tree_mid(M01, g.q, qn));
                    coef[rb_odd + c2] = c;
                    if (frow) frow[2 * (uint64_t)c2 + 1] = c;
                    K kk = abs_key(c);
                    mk = kk > mk ? kk : mk;
                }
            }
            load(k + D, ring[d]);
        }
    }
}

template <class T>
__device__ __forceinline__ void decompose_row_odd_any(const T* __restrict__ in, uint64_t s0, uint64_t s1,
                                                      const Box& F, const Box& C, T* __restrict__ coef,
                                                      T* __restrict__ coarse, T* __restrict__ fnat, uint32_t row,
                                                      uint32_t lane, typename KeyOf<T>::type& mk,
                                                      typename KeyOf<T>::type& mc) {
    const uint32_t c2n = C.n[2];
    const uint32_t x0 = row / F.n[1], x1 = row - x0 * F.n[1];
    const int m01 = (is_coarse(x0, F.n[0]) ? 0 : 1) | (is_coarse(x1, F.n[1]) ? 0 : 2);
    const uint32_t r0 = reord(x0, F.n[0], C.n[0]), r1 = reord(x1, F.n[1], C.n[1]);
    bool cc;
    const uint64_t rbase = row_rank_base(r0, r1, F, C, cc);
    // even node 2c: rank rbase + c (cc rows have none); odd node: rbase + c (cc) or rbase + c2n + c
    const uint64_t rb_even = rbase, rb_odd = cc ? rbase : rbase + c2n;
    const T* p = in + x0 * s0 + x1 * s1;
    T* frow = fnat ? fnat + (uint64_t)row * F.n[2] : nullptr;
    T* crow = coarse + ((uint64_t)r0 * C.n[1] + r1) * c2n;
    switch (m01) {
        case 0: decompose_row_odd<T, 0>(p, s0, s1, c2n, coef, rb_even, rb_odd, crow, frow, lane, mk, mc); break;
        case 1: decompose_row_odd<T, 1>(p, s0, s1, c2n, coef, rb_even, rb_odd, crow, frow, lane, mk, mc); break;
        case 2: decompose_row_odd<T, 2>(p, s0, s1, c2n, coef, rb_even, rb_odd, crow, frow, lane, mk, mc); break;
        default: decompose_row_odd<T, 3>(p, s0, s1, c2n, coef, rb_even, rb_odd, crow, frow, lane, mk, mc); break;
    }
}

template <class T, int M01>
__device__ __forceinline__ void recompose_row_odd_g(const T* __restrict__ cb0, uint64_t cs0, uint64_t cs1,
                                                    uint32_t c2n, const T* __restrict__ coef, uint64_t rb_even,
                                                    uint64_t rb_odd, T* __restrict__ orow, uint32_t lane) {
    constexpr int NQ = M01 == 0 ? 1 : (M01 == 3 ? 4 : 2);
    constexpr int D = M01 == 3 ? 3 : 4;
    int64_t co[4];
    corner_offsets(M01, 0, (int64_t)cs0, 0, (int64_t)cs1, co);
    struct G { T ce, cod, q[NQ]; };
    auto load = [&](uint32_t k, G& g) {
        const uint32_t c = 32 * k + lane;
        const bool a = c < c2n, o = c + 1 < c2n;
#pragma unroll
        for (int i = 0; i < NQ; i++) g.q[i] = a ? __ldg(cb0 + c + co[i]) : (T)0;
        g.ce = (M01 != 0 && a) ? __ldg(coef + rb_even + c) : (T)0;
        g.cod = o ? __ldg(coef + rb_odd + c) : (T)0;
    };
    const uint32_t groups = (c2n + 31) / 32;
    G ring[D];
#pragma unroll
    for (int d = 0; d < D; d++) load(d, ring[d]);
    for (uint32_t k0 = 0; k0 < groups; k0 += D) {
#pragma unroll
        for (int d = 0; d < D; d++) {
            const uint32_t k = k0 + d;
            if (k >= groups) break;
            const G& g = ring[d];
            const G& gx = ring[(d + 1) % D];
            T qn[NQ];
#pragma unroll
            for (int i = 0; i < NQ; i++) qn[i] = __shfl_sync(0xffffffffu, lane == 0 ? gx.q[i] : g.q[i], (lane + 1) & 31);
            const uint32_t c2 = 32 * k + lane;
            if (c2 < c2n) {
                T* o = orow + 2 * (uint64_t)c2;
                o[0] = M01 == 0 ? g.q[0] : add_rn(g.ce, corner_tree(M01, g.q));
                if (c2 + 1 < c2n) o[1] = add_rn(g.cod, corner_tree_mid(M01, g.q, qn));
            }
            load(k + D, ring[d]);
        }
    }
}

template <class T>
__device__ __forceinline__ void recompose_row_odd_any(const T* __restrict__ coarse, const T* __restrict__ coef,
                                                      const Box& F, const Box& C, T* __restrict__ out, uint64_t s0,
                                                      uint64_t s1, uint32_t row, uint32_t lane) {
    const uint32_t c2n = C.n[2];
    const uint64_t cs0 = (uint64_t)C.n[1] * C.n[2], cs1 = C.n[2];
    const uint32_t x0 = row / F.n[1], x1 = row - x0 * F.n[1];
    const int m01 = (is_coarse(x0, F.n[0]) ? 0 : 1) | (is_coarse(x1, F.n[1]) ? 0 : 2);
    const uint32_t r0 = reord(x0, F.n[0], C.n[0]), r1 = reord(x1, F.n[1], C.n[1]);
    const uint32_t c0 = (m01 & 1) ? (x0 >> 1) : r0;
    const uint32_t c1 = (m01 & 2) ? (x1 >> 1) : r1;
    bool cc;
    const uint64_t rbase = row_rank_base(r0, r1, F, C, cc);
    const uint64_t rb_even = rbase, rb_odd = cc ? rbase : rbase + c2n;
    const T* cb0 = coarse + c0 * cs0 + c1 * cs1;
    T* orow = out + x0 * s0 + x1 * s1;
    switch (m01) {
        case 0: recompose_row_odd_g<T, 0>(cb0, cs0, cs1, c2n, coef, rb_even, rb_odd, orow, lane); break;
        case 1: recompose_row_odd_g<T, 1>(cb0, cs0, cs1, c2n, coef, rb_even, rb_odd, orow, lane); break;
        case 2: recompose_row_odd_g<T, 2>(cb0, cs0, cs1, c2n, coef, rb_even, rb_odd, orow, lane); break;
        default: recompose_row_odd_g<T, 3>(cb0, cs0, cs1, c2n, coef, rb_even, rb_odd, orow, lane); break;
    }
}

// inverse level on fine row `row`: coarse box + coefficients -> out row
template <class T>
__device__ __forceinline__ void recompose_row(const T* __restrict__ coarse, const T* __restrict__ coef, const Box& F,
                                              const Box& C, T* __restrict__ out, uint64_t s0, uint64_t s1,
                                              uint32_t row, uint32_t lane) {
    const uint32_t n2 = F.n[2], c2n = C.n[2];
    const uint64_t cs0 = (uint64_t)C.n[1] * C.n[2], cs1 = C.n[2];
    const uint32_t x0 = row / F.n[1], x1 = row - x0 * F.n[1];
    const int m01 = (is_coarse(x0, F.n[0]) ? 0 : 1) | (is_coarse(x1, F.n[1]) ? 0 : 2);
    const uint32_t c0 = (m01 & 1) ? (x0 >> 1) : reord(x0, F.n[0], C.n[0]);
    const uint32_t c1 = (m01 & 2) ? (x1 >> 1) : reord(x1, F.n[1], C.n[1]);
    const uint32_t r0 = reord(x0, F.n[0], C.n[0]), r1 = reord(x1, F.n[1], C.n[1]);
    bool cc;
    const uint64_t rbase = row_rank_base(r0, r1, F, C, cc);
    const T* cb0 = coarse + c0 * cs0 + c1 * cs1;
    int64_t co[4];
    corner_offsets(m01, 0, (int64_t)cs0, 0, (int64_t)cs1, co);
    const int nq = corner_count(m01);
    T* orow = out + x0 * s0 + x1 * s1;
#pragma unroll 3
    for (uint32_t cbase = 0; cbase < c2n; cbase += 32) {
        const uint32_t c2 = cbase + lane;
        const bool act = c2 < c2n;
        const bool odd = act && c2 + 1 < c2n && fine_of_coarse(c2 + 1, n2, c2n) == 2 * c2 + 2;
        T q[4] = {0, 0, 0, 0}, qn[4];
#pragma unroll
        for (int i = 0; i < 4; i++)
            if (i < nq && act) q[i] = __ldg(cb0 + c2 + co[i]);
#pragma unroll
        for (int i = 0; i < 4; i++) {
            qn[i] = __shfl_down_sync(0xffffffffu, q[i], 1);
            if (i < nq && lane == 31 && odd) qn[i] = __ldg(cb0 + c2 + 1 + co[i]);
        }
        if (act) {
            const uint32_t xe = fine_of_coarse(c2, n2, c2n);
            orow[xe] = m01 == 0 ? q[0] : add_rn(coef[rbase + (cc ? c2 - c2n : c2)], corner_tree(m01, q));
            if (odd) orow[2 * c2 + 1] = add_rn(coef[rbase + (cc ? c2 : c2n + c2)], corner_tree_mid(m01, q, qn));
        }
    }
}

}  // namespace prodm
