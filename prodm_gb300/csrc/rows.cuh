// Per-row bodies of the row-parallel MGARD kernels (one warp per fine row),
// shared by the single-field kernels and the multi-field batched kernels.
#pragma once
#include <cstdlib>
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

// ---------------------------------------------------------------------------
// Patch form of the decomposition for grids whose every dim is 2 C - 1 (the
// 2^k + 1 grids): a warp takes coarse columns c = 32 g + lane of the fine
// rows x0 in {2i, 2i+1} x x1 in {2b, 2b+1} for kPatchSteps consecutive b.
// With q the fine values at even x2 (the corner nodes) of the rows 2i, 2i+2
// (x0) and 2b, 2b+2 (x1), h = avg(q at 2c, q at 2c+2), the four rows' nodes
// 2c, 2c+1 subtract
//   (2i,   2b  ): -        | h00                 (even node: coarse node)
//   (2i,   2b+1): V0       | HV0                 V0 = avg(q00, q02), HV0 = avg(h00, h02)
//   (2i+1, 2b  ): avg(q00, q20)  | avg(h00, h20)
//   (2i+1, 2b+1): avg(V0, V2)    | avg(HV0, HV2)  V2 = avg(q20, q22), HV2 = avg(h20, h22)
// -- the row kernels' corner trees (dim 2 innermost, dim 0 outermost), so the
// coefficients are bit-identical to decompose_row_odd's. Each interpolation
// is formed once per 2 x 2 rows and the corner rows 2b + 2 carry over to the
// next b. The last node of each row (x2 = F2 - 1, even only) is taken by the
// lane holding coarse column P = C2 - 1 (or, when P is a multiple of 32, by
// lane 31 of the last group, from the neighbour values it loads itself).
// ---------------------------------------------------------------------------
constexpr uint32_t kPatchSteps = 8;

__host__ __device__ inline bool patch_grid(const Box& F, const Box& C) {
    return F.n[0] == 2 * C.n[0] - 1 && F.n[1] == 2 * C.n[1] - 1 && F.n[2] == 2 * C.n[2] - 1 && C.n[2] >= 2;
}
// warp items of one level: slabs x strips x column groups
__host__ __device__ inline uint64_t patch_items(const Box& C) {
    const uint32_t npg = (C.n[2] - 1 + 31) >> 5;
    return (uint64_t)C.n[0] * ((C.n[1] + kPatchSteps - 1) / kPatchSteps) * npg;
}
// a level takes the patch kernels when it is a patch grid with enough items:
// each item walks kPatchSteps steps one after another, so a small level (a
// few hundred items) runs faster as one warp per row (at 513^3 levels 7 and 6
// have 67,848 and 8,772 items; level 5 has 1,170). The threshold is 2048
// items, or PRODM_PATCH_MIN_ITEMS (read at each use; the tests set 1 to run
// the patch kernels on small grids).
inline uint64_t patch_min_items() {
    const char* v = getenv("PRODM_PATCH_MIN_ITEMS");
    return v ? strtoull(v, nullptr, 10) : 2048ull;
}
inline bool patch_level(const Box& F, const Box& C) {
    return patch_grid(F, C) && patch_items(C) >= patch_min_items();
}

template <class T>
__device__ __forceinline__ void decompose_patch_item(const T* __restrict__ in, uint64_t s0, uint64_t s1,
                                                     const Box& F, const Box& C, T* __restrict__ coef,
                                                     T* __restrict__ coarse, uint64_t item, uint32_t lane,
                                                     typename KeyOf<T>::type& mk, typename KeyOf<T>::type& mc) {
    using K = typename KeyOf<T>::type;
    const uint32_t C0 = C.n[0], C1 = C.n[1], C2 = C.n[2];
    const uint32_t P = C2 - 1, npg = (P + 31) >> 5, nstrip = (C1 + kPatchSteps - 1) / kPatchSteps;
    const uint32_t g = (uint32_t)(item % npg);
    const uint64_t r = item / npg;
    const uint32_t u = (uint32_t)(r % nstrip), i = (uint32_t)(r / nstrip);
    const uint32_t c = 32 * g + lane;
    const bool act = c < P;                        // a column pair (2c, 2c+1)
    const bool ld = c <= P;                        // holds coarse column c
    const bool two = i + 1 < C0;                   // fine row 2i + 1 exists
    // the last node: its own column (P not a multiple of 32) or lane 31's neighbour
    const bool last = (g == npg - 1) && ((P & 31) ? (lane == (P & 31)) : (lane == 31));
    const bool own = c == P;
    const uint32_t b0 = u * kPatchSteps, b1 = min(b0 + kPatchSteps, C1);
    const T* base = in + (uint64_t)(2 * i) * s0;
    auto kmax = [](K& m, T v) { const K k = abs_key(v); m = k > m ? k : m; };
    // the loads of one step, issued a step ahead of their use: the four
    // rows' node pairs, the corner values of rows 2b + 2 at column c and (lane
    // 31) at column c + 1, and the last node's even values
    struct Step {
        T a00, e01, o01, e10, o10, e11, o11, q02, q22, n02, n22, l01, l10, l11;
    };
    auto load_step = [&](uint32_t b, Step& S) {
        const bool odd = b + 1 < C1;
        const T* r00 = base + (uint64_t)(2 * b) * s1;
        const T* r01 = r00 + s1;
        const T* r10 = r00 + s0;
        const T* r11 = r10 + s1;
        const uint64_t x = 2 * (uint64_t)c, xl = 2 * (uint64_t)P;
        S.a00 = act ? r00[x + 1] : (T)0;
        S.e01 = act && odd ? r01[x] : (T)0;
        S.o01 = act && odd ? r01[x + 1] : (T)0;
        S.e10 = act && two ? r10[x] : (T)0;
        S.o10 = act && two ? r10[x + 1] : (T)0;
        S.e11 = act && two && odd ? r11[x] : (T)0;
        S.o11 = act && two && odd ? r11[x + 1] : (T)0;
        S.q02 = ld && odd ? r00[2 * s1 + x] : (T)0;
        S.q22 = ld && odd && two ? r00[2 * s0 + 2 * s1 + x] : (T)0;
        S.n02 = lane == 31 && act && odd ? r00[2 * s1 + x + 2] : (T)0;
        S.n22 = lane == 31 && act && odd && two ? r00[2 * s0 + 2 * s1 + x + 2] : (T)0;
        S.l01 = last && odd ? r01[xl] : (T)0;
        S.l10 = last && two ? r10[xl] : (T)0;
        S.l11 = last && two && odd ? r11[xl] : (T)0;
    };
    // corner values at column c + 1: the next lane's, lane 31's own load
    auto next_col = [&](T q, T own_next) {
        const T n = __shfl_down_sync(0xffffffffu, q, 1);
        return lane == 31 ? own_next : n;
    };
    T q00, q20 = 0;
    {
        const T* r = base + (uint64_t)(2 * b0) * s1;
        const uint64_t x = 2 * (uint64_t)c;
        q00 = ld ? r[x] : (T)0;
        T n00 = lane == 31 && act ? r[x + 2] : (T)0, n20 = 0;
        if (two) {
            q20 = ld ? r[2 * s0 + x] : (T)0;
            n20 = lane == 31 && act ? r[2 * s0 + x + 2] : (T)0;
        }
        n00 = next_col(q00, n00);
        n20 = next_col(q20, n20);
        Step S;
        load_step(b0, S);
        T qn00 = n00, qn20 = n20;
        T h00 = avg_rn(q00, qn00), h20 = avg_rn(q20, qn20);
        for (uint32_t b = b0; b < b1; b++) {
            Step Sn = S;
            if (b + 1 < b1) load_step(b + 1, Sn);
            const bool odd = b + 1 < C1;
            const T qn02 = next_col(S.q02, S.n02), qn22 = next_col(S.q22, S.n22);
            const T q02 = S.q02, q22 = S.q22;
            const T h02 = avg_rn(q02, qn02), h22 = avg_rn(q22, qn22);
            const uint64_t rb00 = level_rank(i, b, C2, F, C);              // even-even row: odd nodes only
            const uint64_t rb01 = level_rank(i, C1 + b, 0, F, C);
            const uint64_t rb10 = level_rank(C0 + i, b, 0, F, C);
            const uint64_t rb11 = level_rank(C0 + i, C1 + b, 0, F, C);
            T* crow = coarse + ((uint64_t)i * C1 + b) * C2;
            const T v0 = avg_rn(q00, q02), hv0 = avg_rn(h00, h02);
            const T v2 = avg_rn(q20, q22), hv2 = avg_rn(h20, h22);
            if (act) {
                crow[c] = q00;
                kmax(mc, q00);
                T d = sub_rn(S.a00, h00);
                coef[rb00 + c] = d;
                kmax(mk, d);
                if (odd) {
                    d = sub_rn(S.e01, v0);
                    coef[rb01 + c] = d;
                    kmax(mk, d);
                    d = sub_rn(S.o01, hv0);
                    coef[rb01 + C2 + c] = d;
                    kmax(mk, d);
                }
                if (two) {
                    d = sub_rn(S.e10, avg_rn(q00, q20));
                    coef[rb10 + c] = d;
                    kmax(mk, d);
                    d = sub_rn(S.o10, avg_rn(h00, h20));
                    coef[rb10 + C2 + c] = d;
                    kmax(mk, d);
                    if (odd) {
                        d = sub_rn(S.e11, avg_rn(v0, v2));
                        coef[rb11 + c] = d;
                        kmax(mk, d);
                        d = sub_rn(S.o11, avg_rn(hv0, hv2));
                        coef[rb11 + C2 + c] = d;
                        kmax(mk, d);
                    }
                }
            }
            if (last) {   // coarse column P: the rows' last (even) nodes
                const T p00 = own ? q00 : qn00, p02 = own ? q02 : qn02;
                const T p20 = own ? q20 : qn20, p22 = own ? q22 : qn22;
                crow[P] = p00;
                kmax(mc, p00);
                const T w0 = avg_rn(p00, p02);
                if (odd) {
                    const T d = sub_rn(S.l01, w0);
                    coef[rb01 + P] = d;
                    kmax(mk, d);
                }
                if (two) {
                    T d = sub_rn(S.l10, avg_rn(p00, p20));
                    coef[rb10 + P] = d;
                    kmax(mk, d);
                    if (odd) {
                        d = sub_rn(S.l11, avg_rn(w0, avg_rn(p20, p22)));
                        coef[rb11 + P] = d;
                        kmax(mk, d);
                    }
                }
            }
            q00 = q02;
            qn00 = qn02;
            h00 = h02;
            q20 = q22;
            qn20 = qn22;
            h20 = h22;
            S = Sn;
        }
    }
}

// Patch form of the recomposition (the inverse of decompose_patch_item): the
// same warp items; the corner values come from the compact coarse box (rows
// (i, b), (i, b+1), (i+1, b), (i+1, b+1) of its coarse columns), the
// coefficients from the packed level, and the four fine rows' nodes 2c, 2c+1
// are the coefficient plus the interpolation of decompose_patch_item (the
// row kernels' corner trees, so the output is bit-identical to theirs). Each
// step's loads are issued a step ahead of their use.
template <class T>
__device__ __forceinline__ void recompose_patch_item(const T* __restrict__ coarse, const T* __restrict__ coef,
                                                     const Box& F, const Box& C, T* __restrict__ out, uint64_t s0,
                                                     uint64_t s1, uint64_t item, uint32_t lane) {
    const uint32_t C0 = C.n[0], C1 = C.n[1], C2 = C.n[2];
    const uint32_t P = C2 - 1, npg = (P + 31) >> 5, nstrip = (C1 + kPatchSteps - 1) / kPatchSteps;
    const uint32_t g = (uint32_t)(item % npg);
    const uint64_t r = item / npg;
    const uint32_t u = (uint32_t)(r % nstrip), i = (uint32_t)(r / nstrip);
    const uint32_t c = 32 * g + lane;
    const bool act = c < P;
    const bool ld = c <= P;
    const bool two = i + 1 < C0;
    const bool last = (g == npg - 1) && ((P & 31) ? (lane == (P & 31)) : (lane == 31));
    const bool own = c == P;
    const uint32_t b0 = u * kPatchSteps, b1 = min(b0 + kPatchSteps, C1);
    const uint64_t cs0 = (uint64_t)C1 * C2;
    const T* slab0 = coarse + (uint64_t)i * cs0;         // coarse rows (i, b)
    const T* slab1 = slab0 + cs0;                         // (i + 1, b)
    struct Step {
        T q02, q22, n02, n22, ca, cbe, cbo, cce, cco, cde, cdo, lb, lc, ld_;
    };
    auto load_step = [&](uint32_t b, Step& S) {
        const bool odd = b + 1 < C1;
        const uint64_t rb00 = level_rank(i, b, C2, F, C);
        const uint64_t rb01 = level_rank(i, C1 + b, 0, F, C);
        const uint64_t rb10 = level_rank(C0 + i, b, 0, F, C);
        const uint64_t rb11 = level_rank(C0 + i, C1 + b, 0, F, C);
        const T* q0 = slab0 + (uint64_t)(b + 1) * C2;
        const T* q1 = slab1 + (uint64_t)(b + 1) * C2;
        S.q02 = ld && odd ? __ldg(q0 + c) : (T)0;
        S.q22 = ld && odd && two ? __ldg(q1 + c) : (T)0;
        S.n02 = lane == 31 && act && odd ? __ldg(q0 + c + 1) : (T)0;
        S.n22 = lane == 31 && act && odd && two ? __ldg(q1 + c + 1) : (T)0;
        S.ca = act ? __ldg(coef + rb00 + c) : (T)0;
        S.cbe = act && odd ? __ldg(coef + rb01 + c) : (T)0;
        S.cbo = act && odd ? __ldg(coef + rb01 + C2 + c) : (T)0;
        S.cce = act && two ? __ldg(coef + rb10 + c) : (T)0;
        S.cco = act && two ? __ldg(coef + rb10 + C2 + c) : (T)0;
        S.cde = act && two && odd ? __ldg(coef + rb11 + c) : (T)0;
        S.cdo = act && two && odd ? __ldg(coef + rb11 + C2 + c) : (T)0;
        S.lb = last && odd ? __ldg(coef + rb01 + P) : (T)0;
        S.lc = last && two ? __ldg(coef + rb10 + P) : (T)0;
        S.ld_ = last && two && odd ? __ldg(coef + rb11 + P) : (T)0;
    };
    auto next_col = [&](T q, T own_next) {
        const T n = __shfl_down_sync(0xffffffffu, q, 1);
        return lane == 31 ? own_next : n;
    };
    const T* q0 = slab0 + (uint64_t)b0 * C2;
    const T* q1 = slab1 + (uint64_t)b0 * C2;
    T q00 = ld ? __ldg(q0 + c) : (T)0, q20 = ld && two ? __ldg(q1 + c) : (T)0;
    T qn00 = next_col(q00, lane == 31 && act ? __ldg(q0 + c + 1) : (T)0);
    T qn20 = next_col(q20, lane == 31 && act && two ? __ldg(q1 + c + 1) : (T)0);
    T h00 = avg_rn(q00, qn00), h20 = avg_rn(q20, qn20);
    Step S;
    load_step(b0, S);
    for (uint32_t b = b0; b < b1; b++) {
        Step Sn = S;
        if (b + 1 < b1) load_step(b + 1, Sn);
        const bool odd = b + 1 < C1;
        const T q02 = S.q02, q22 = S.q22;
        const T qn02 = next_col(q02, S.n02), qn22 = next_col(q22, S.n22);
        const T h02 = avg_rn(q02, qn02), h22 = avg_rn(q22, qn22);
        const T v0 = avg_rn(q00, q02), hv0 = avg_rn(h00, h02);
        const T v2 = avg_rn(q20, q22), hv2 = avg_rn(h20, h22);
        T* o00 = out + (uint64_t)(2 * i) * s0 + (uint64_t)(2 * b) * s1;
        T* o01 = o00 + s1;
        T* o10 = o00 + s0;
        T* o11 = o10 + s1;
        if (act) {
            const uint64_t x = 2 * (uint64_t)c;
            o00[x] = q00;
            o00[x + 1] = add_rn(S.ca, h00);
            if (odd) {
                o01[x] = add_rn(S.cbe, v0);
                o01[x + 1] = add_rn(S.cbo, hv0);
            }
            if (two) {
                o10[x] = add_rn(S.cce, avg_rn(q00, q20));
                o10[x + 1] = add_rn(S.cco, avg_rn(h00, h20));
                if (odd) {
                    o11[x] = add_rn(S.cde, avg_rn(v0, v2));
                    o11[x + 1] = add_rn(S.cdo, avg_rn(hv0, hv2));
                }
            }
        }
        if (last) {   // coarse column P: the rows' last (even) nodes
            const uint64_t x = 2 * (uint64_t)P;
            const T p00 = own ? q00 : qn00, p02 = own ? q02 : qn02;
            const T p20 = own ? q20 : qn20, p22 = own ? q22 : qn22;
            o00[x] = p00;
            const T w0 = avg_rn(p00, p02);
            if (odd) o01[x] = add_rn(S.lb, w0);
            if (two) {
                o10[x] = add_rn(S.lc, avg_rn(p00, p20));
                if (odd) o11[x] = add_rn(S.ld_, avg_rn(w0, avg_rn(p20, p22)));
            }
        }
        q00 = q02;
        qn00 = qn02;
        h00 = h02;
        q20 = q22;
        qn20 = qn22;
        h20 = h22;
        S = Sn;
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
