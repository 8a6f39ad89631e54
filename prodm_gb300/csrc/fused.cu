// Fused finest-level retrieval (sm_103a): negabinary decode of the level's
// retrieved planes + hierarchical recomposition, in one pass.
//
// The unfused path writes the decoded level coefficients (n_L values) and
// reads them back in the recomposition; at the finest level that is most of
// the field. Here one warp owns one fine row (x0, x1): the coefficients of a
// row occupy one contiguous run of interleaved ranks, so the warp decodes the
// 32-value blocks covering that run (one bit transpose per block) into shared
// memory and then writes the recomposed row with coalesced stores. Decoding
// and recomposition use exactly the arithmetic of the standalone kernels
// (NegaBinaryBPEncoder.hpp:132-192; the multilinear interpolation of the
// hierarchical basis), so the output is bit-identical to the unfused path.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <cstdlib>
#include <mutex>

#include "common.cuh"
#include "kernels.cuh"
#include "nbcodec.cuh"

namespace prodm {

namespace {

constexpr unsigned FULL = 0xffffffffu;

// ---------------------------------------------------------------------------
// TMA (cp.async.bulk.tensor) + mbarrier helpers
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
// this thread's arrival plus `bytes` more expected from asynchronous copies
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// waits for the phase with this parity at most `limit` SM clock cycles
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, long long limit) {
    const long long t0 = clock64();
    while (!mbar_try_wait(bar, parity))
        if (clock64() - t0 > limit) return false;
    return true;
}
// this thread's arrival (release of its earlier shared-memory writes)
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar)) : "memory");
}
// named barrier 1 over the first `n` threads of the block
__device__ __forceinline__ void group_sync(int n) { asm volatile("bar.sync 1, %0;" ::"r"(n) : "memory"); }
// generic-proxy accesses of shared memory before async-proxy (TMA) ones
__device__ __forceinline__ void fence_proxy_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
// box {x .. x + box_w - 1} of row y of a 2-D tensor map into shared memory
__device__ __forceinline__ void tma_load_2d(uint32_t* dst, const CUtensorMap* map, int x, int y, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];"
        ::"r"(smem_addr(dst)), "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_addr(bar))
        : "memory");
}

__device__ __forceinline__ float pow2f_(int e) { return __int_as_float((e + 127) << 23); }

__device__ __forceinline__ uint32_t natural_of(uint32_t r, uint32_t n, uint32_t nc) {
    return r < nc ? fine_of_coarse(r, n, nc) : 2 * (r - nc) + 1;
}

// CTA = 8 warps = 8 consecutive rows in the reordered (interleaved-rank)
// order, so the CTA's coefficients form one contiguous rank range: the CTA
// stages the retrieved planes of that range in shared memory with coalesced
// loads, decodes them (one transpose per 32-value block) into a shared
// coefficient buffer, then each warp writes its natural-order output row.
__global__ void __launch_bounds__(256) k_decode_recompose_nb32(const uint32_t* __restrict__ base, uint64_t stride,
                                                              const uint32_t* __restrict__ maxkey,
                                                              const uint8_t* __restrict__ dnum,
                                                              const float* __restrict__ coarse, Box F, Box C,
                                                              float* __restrict__ out, uint64_t s0, uint64_t s1,
                                                              uint32_t max_blocks) {
    extern __shared__ uint32_t smem[];
    uint32_t* tile = smem;                                   // [plane][max_blocks]
    const uint32_t pad = max_blocks | 1u;                    // odd row length: conflict-free
    float* cbuf = (float*)(smem + 32 * max_blocks);          // [32][pad]
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int num = dnum[0];
    const int exp = frexp_exp(__uint_as_float(*maxkey)) + 2;
    const int e = num;
    const bool neg = num != 0 && (e & 1);
    const bool dfast = (exp - e) >= -126 && (exp - e) <= 127;
    const float dscale = dfast ? pow2f_(exp - e) : 1.f;
    const uint32_t rows = F.n[0] * F.n[1];
    const uint32_t n2 = F.n[2], c2n = C.n[2];
    const uint64_t cs0 = (uint64_t)C.n[1] * C.n[2], cs1 = C.n[2];
    auto row_info = [&](uint32_t rho, uint32_t& r0, uint32_t& r1, bool& cc, uint64_t& rbase, uint32_t& len) {
        r0 = rho / F.n[1];
        r1 = rho - r0 * F.n[1];
        cc = r0 < C.n[0] && r1 < C.n[1];
        rbase = level_rank(r0, r1, cc ? c2n : 0u, F, C);
        len = cc ? n2 - c2n : n2;
    };
    for (uint32_t rho0 = blockIdx.x * 8; rho0 < rows; rho0 += gridDim.x * 8) {
        const uint32_t rho_last = min(rho0 + 7, rows - 1);
        uint32_t a0, a1, z0, z1, alen, zlen;
        bool acc_, zcc;
        uint64_t abase, zbase;
        row_info(rho0, a0, a1, acc_, abase, alen);
        row_info(rho_last, z0, z1, zcc, zbase, zlen);
        const uint64_t fb = abase >> 5, lb = (zbase + zlen - 1) >> 5;
        const uint32_t nbk = (uint32_t)(lb - fb + 1);
        // stage the planes of blocks [fb, lb]
        for (int p = warp; p < num; p += 8) {
            const uint32_t* src = base + (uint64_t)p * stride + fb;
            uint32_t* row = tile + p * max_blocks;
            for (uint32_t j = lane; j < nbk; j += 32) row[j] = __ldcs(src + j);
        }
        __syncthreads();
        // one thread per 32-value block: register transpose of the block's
        // plane words; value e of block t goes to cbuf[e * pad + t]
        for (uint32_t t = threadIdx.x; t < nbk; t += blockDim.x) {
            uint32_t a[32];
#pragma unroll
            for (int p = 0; p < 32; p++) a[p] = p < num ? tile[p * max_blocks + t] : 0u;
            transpose32_regs(a);
#pragma unroll
            for (int v = 0; v < 32; v++) {
                const uint32_t acc = num ? (__brev(a[v]) >> (32 - num)) : 0u;
                float val = num ? (dfast ? (float)nb_to_bin(acc) * dscale : ldexpf((float)nb_to_bin(acc), exp - e)) : 0.f;
                cbuf[v * pad + t] = neg ? -val : val;
            }
        }
        __syncthreads();
        const uint32_t rho = rho0 + warp;
        if (rho < rows) {
            uint32_t r0, r1, len;
            bool cc;
            uint64_t rbase;
            row_info(rho, r0, r1, cc, rbase, len);
            const uint32_t x0 = natural_of(r0, F.n[0], C.n[0]), x1 = natural_of(r1, F.n[1], C.n[1]);
            const int m01 = (is_coarse(x0, F.n[0]) ? 0 : 1) | (is_coarse(x1, F.n[1]) ? 0 : 2);
            const uint32_t c0 = (m01 & 1) ? (x0 >> 1) : r0;
            const uint32_t c1 = (m01 & 2) ? (x1 >> 1) : r1;
            const float* cb0 = coarse + c0 * cs0 + c1 * cs1;
            int64_t co[4];
            if (m01 == 0) { co[0] = 0; }
            else if (m01 == 1) { co[0] = 0; co[1] = (int64_t)cs0; }
            else if (m01 == 2) { co[0] = 0; co[1] = (int64_t)cs1; }
            else { co[0] = 0; co[1] = (int64_t)cs1; co[2] = (int64_t)cs0; co[3] = (int64_t)(cs0 + cs1); }
            const int nq = corner_count(m01);
            float* orow = out + x0 * s0 + x1 * s1;
            const uint32_t rb0 = (uint32_t)(rbase - fb * 32);
            auto coefat = [&](uint32_t off) { const uint32_t r = rb0 + off; return cbuf[(r & 31) * pad + (r >> 5)]; };
            for (uint32_t cbase = 0; cbase < c2n; cbase += 32) {
                const uint32_t c2 = cbase + lane;
                const bool act = c2 < c2n;
                const bool odd = act && c2 + 1 < c2n && fine_of_coarse(c2 + 1, n2, c2n) == 2 * c2 + 2;
                float q[4] = {0.f, 0.f, 0.f, 0.f}, qn[4];
#pragma unroll
                for (int i = 0; i < 4; i++)
                    if (i < nq && act) q[i] = __ldg(cb0 + c2 + co[i]);
#pragma unroll
                for (int i = 0; i < 4; i++) {
                    qn[i] = __shfl_down_sync(FULL, q[i], 1);
                    if (i < nq && lane == 31 && odd) qn[i] = __ldg(cb0 + c2 + 1 + co[i]);
                }
                if (act) {
                    const uint32_t xe = fine_of_coarse(c2, n2, c2n);
                    orow[xe] = m01 == 0 ? q[0] : __fadd_rn(coefat(cc ? c2 - c2n : c2), corner_tree(m01, q));
                    if (odd) orow[2 * c2 + 1] = __fadd_rn(coefat(cc ? c2 : c2n + c2), corner_tree_mid(m01, q, qn));
                }
            }
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// Odd row length (n = 2^k + 1 and every other odd n): fine node 2c of a row is
// coarse node c and the odd node 2c+1 lies between coarse nodes c and c+1, so
// the row walk needs no index remapping. The planes of the next 8 rows are
// fetched with cp.async into a second tile while the current rows are decoded
// and recomposed; the coefficient buffer is value-major ([block][33]).
// ---------------------------------------------------------------------------
constexpr int CB_LD = 36;   // value-major coefficient rows: conflict-free both ways

__device__ __forceinline__ float cb_at(const float* cb, uint32_t r) { return cb[(r >> 5) * CB_LD + (r & 31)]; }

// one fine row of odd length n = 2 c2n - 1; M01 = odd-dim mask over dims
// 0/1 (0: both coarse -> only odd nodes carry coefficients, ranks c;
// otherwise even node 2c has rank c and odd node 2c+1 rank c2n + c). The row
// is c2n - 1 column pairs (nodes 2c, 2c+1) and a last node 2(c2n - 1). Lane l
// handles the pairs 32k + l; the corner values of D column groups are in
// flight at once (a ring of D groups in registers, refilled as each group is
// used), so a row waits for the L2 latency about once instead of once per
// group. Groups in which every lane has a pair run without bounds checks, on
// pointers advanced once per D groups; the last node is written by lane 0.
template <int M01, bool DEEP = false>
__device__ __forceinline__ void recompose_row_odd(const float* __restrict__ cb0, uint64_t cs0, uint64_t cs1,
                                                  uint32_t c2n, const float* __restrict__ cb, uint32_t rb0,
                                                  float* __restrict__ orow, int lane) {
    constexpr int NQ = M01 == 0 ? 1 : (M01 == 3 ? 4 : 2);
    constexpr int D = DEEP ? (M01 == 3 ? 4 : 6) : (M01 == 3 ? 3 : 4);   // column groups in flight
    int64_t co[NQ];   // corner row offsets, in corner_tree order
    co[0] = 0;
    if constexpr (NQ == 2) co[1] = (int64_t)(M01 == 1 ? cs0 : cs1);
    if constexpr (NQ == 4) {
        co[1] = (int64_t)cs1;
        co[2] = (int64_t)cs0;
        co[3] = (int64_t)(cs0 + cs1);
    }
    const uint32_t P = c2n - 1;
    if (lane == 0) {   // the last node: coarse column P
        float q[NQ];
#pragma unroll
        for (int i = 0; i < NQ; i++) q[i] = __ldg(cb0 + P + co[i]);
        if constexpr (M01 == 0) orow[2 * (uint64_t)P] = q[0];
        else orow[2 * (uint64_t)P] = __fadd_rn(cb_at(cb, rb0 + P), corner_tree(M01, q));
    }
    if (P == 0) return;
    const float* pc[NQ];
#pragma unroll
    for (int i = 0; i < NQ; i++) pc[i] = cb0 + co[i] + lane;
    // coefficient of rank r at cb[r + (r >> 5)]: 33 floats further per 32 ranks
    const uint32_t re = rb0 + lane, ro = rb0 + (M01 == 0 ? 0u : c2n) + lane;
    const float* pe = cb + (re >> 5) * CB_LD + (re & 31);
    const float* po = cb + (ro >> 5) * CB_LD + (ro & 31);
    float* o = orow + 2 * lane;
    const int lim = (int)c2n - lane;   // column 32k + lane exists <=> 32k < lim
    const uint32_t groups = (P + 31) >> 5, full = P >> 5;
    float ring[D][NQ];
#pragma unroll
    for (int d = 0; d < D; d++)
#pragma unroll
        for (int i = 0; i < NQ; i++) ring[d][i] = 32 * d < lim ? __ldg(pc[i] + 32 * d) : 0.f;
    const int src = (lane + 1) & 31;
    auto pair = [&](const float (&q)[NQ], const float (&qn)[NQ], const float* e, const float* od, float* out) {
        if constexpr (M01 == 0) {
            out[0] = q[0];
            out[1] = __fadd_rn(*od, avg_rn(q[0], qn[0]));
        } else if constexpr (M01 == 3) {
            out[0] = __fadd_rn(*e, avg_rn(avg_rn(q[0], q[1]), avg_rn(q[2], q[3])));
            out[1] = __fadd_rn(*od, avg_rn(avg_rn(avg_rn(q[0], qn[0]), avg_rn(q[1], qn[1])),
                                           avg_rn(avg_rn(q[2], qn[2]), avg_rn(q[3], qn[3]))));
        } else {
            out[0] = __fadd_rn(*e, avg_rn(q[0], q[1]));
            out[1] = __fadd_rn(*od, avg_rn(avg_rn(q[0], qn[0]), avg_rn(q[1], qn[1])));
        }
    };
    uint32_t k0 = 0;
    for (; k0 + D <= full; k0 += D) {
#pragma unroll
        for (int d = 0; d < D; d++) {
            const float(&q)[NQ] = ring[d];
            const float(&qx)[NQ] = ring[(d + 1) % D];   // group k + 1
            // lane l < 31 takes column c+1 from lane l+1; lane 31 from lane 0 of group k+1
            float qn[NQ];
#pragma unroll
            for (int i = 0; i < NQ; i++) qn[i] = __shfl_sync(FULL, lane == 0 ? qx[i] : q[i], src);
            pair(q, qn, pe + CB_LD * d, po + CB_LD * d, o + 64 * d);
            // refill: group k + D (a slot past the row keeps stale values, never used)
            if ((int)(32 * (k0 + d + D)) < lim) {
#pragma unroll
                for (int i = 0; i < NQ; i++) ring[d][i] = __ldg(pc[i] + 32 * (d + D));
            }
        }
#pragma unroll
        for (int i = 0; i < NQ; i++) pc[i] += 32 * D;
        pe += CB_LD * D;
        po += CB_LD * D;
        o += 64 * D;
    }
    // the remaining groups: fewer than D complete ones and at most one partial
    const int plim = (int)P - lane;   // pair 32k + lane exists <=> 32k < plim
#pragma unroll
    for (int d = 0; d < D; d++) {
        const uint32_t k = k0 + d;
        if (k >= groups) break;
        const float(&q)[NQ] = ring[d];
        const float(&qx)[NQ] = ring[(d + 1) % D];
        float qn[NQ];
#pragma unroll
        for (int i = 0; i < NQ; i++) qn[i] = __shfl_sync(FULL, lane == 0 ? qx[i] : q[i], src);
        if ((int)(32 * k) < plim) pair(q, qn, pe + CB_LD * d, po + CB_LD * d, o + 64 * d);
        if ((int)(32 * (k + D)) < lim) {
#pragma unroll
            for (int i = 0; i < NQ; i++) ring[d][i] = __ldg(pc[i] + 32 * (d + D));
        }
    }
}


// reordered row rho of the fine box: its reordered coordinates (r0, r1),
// whether both are coarse (the row then holds only odd nodes), the rank of
// its first coefficient in the level's interleaved order, and its length
__device__ __forceinline__ void fused_row_rank(uint32_t rho, const Box& F, const Box& C, uint32_t& r0, uint32_t& r1,
                                               bool& cc, uint64_t& rbase, uint32_t& len) {
    r0 = rho / F.n[1];
    r1 = rho - r0 * F.n[1];
    cc = r0 < C.n[0] && r1 < C.n[1];
    rbase = level_rank(r0, r1, cc ? C.n[2] : 0u, F, C);
    len = cc ? F.n[2] - C.n[2] : F.n[2];
}

// block range [fb, fb + nbk) of the coefficients of rows [rho0, rho0 + nr)
__device__ __forceinline__ void fused_block_range(uint32_t rho0, uint32_t rows, const Box& F, const Box& C,
                                                  uint64_t& fb, uint32_t& nbk, uint32_t nr = 8) {
    const uint32_t rho_last = min(rho0 + nr - 1, rows - 1);
    uint32_t a0, a1, z0, z1, alen, zlen;
    bool acc_, zcc;
    uint64_t abase, zbase;
    fused_row_rank(rho0, F, C, a0, a1, acc_, abase, alen);
    fused_row_rank(rho_last, F, C, z0, z1, zcc, zbase, zlen);
    fb = abase >> 5;
    nbk = (uint32_t)(((zbase + zlen - 1) >> 5) - fb + 1);
}

// where fine row rho's inputs and output lie: the first coarse corner row
// (element offset in the coarse box), the output row (element offset), the
// rank of its first coefficient relative to block fb, and its odd-dim mask
struct FusedRow {
    uint64_t coarse_off, out_off;
    uint32_t rb;
    int m01;
};
__device__ __forceinline__ FusedRow fused_row(uint32_t rho, const Box& F, const Box& C, uint64_t s0, uint64_t s1,
                                              uint64_t fb) {
    const uint64_t cs0 = (uint64_t)C.n[1] * C.n[2], cs1 = C.n[2];
    uint32_t r0, r1, len;
    bool cc;
    uint64_t rbase;
    fused_row_rank(rho, F, C, r0, r1, cc, rbase, len);
    const uint32_t x0 = natural_of(r0, F.n[0], C.n[0]), x1 = natural_of(r1, F.n[1], C.n[1]);
    FusedRow r;
    r.m01 = (is_coarse(x0, F.n[0]) ? 0 : 1) | (is_coarse(x1, F.n[1]) ? 0 : 2);
    const uint32_t c0 = (r.m01 & 1) ? (x0 >> 1) : r0;
    const uint32_t c1 = (r.m01 & 2) ? (x1 >> 1) : r1;
    r.coarse_off = c0 * cs0 + c1 * cs1;
    r.out_off = x0 * s0 + x1 * s1;
    r.rb = (uint32_t)(rbase - fb * 32);
    return r;
}

// one warp: a fine row (odd length) from the coarse box and the decoded
// coefficients in cb (value v of block t at cb[t * CB_LD + v], block fb first)
template <bool DEEP = false>
__device__ __forceinline__ void recompose_fine_row(const FusedRow& r, const Box& C, const float* __restrict__ coarse,
                                                   float* __restrict__ out, const float* __restrict__ cb, int lane) {
    const uint32_t c2n = C.n[2];
    const uint64_t cs0 = (uint64_t)C.n[1] * C.n[2], cs1 = C.n[2];
    const float* cb0 = coarse + r.coarse_off;
    float* orow = out + r.out_off;
    const uint32_t rb0 = r.rb;
    switch (r.m01) {
        case 0: recompose_row_odd<0, DEEP>(cb0, cs0, cs1, c2n, cb, rb0, orow, lane); break;
        case 1: recompose_row_odd<1, DEEP>(cb0, cs0, cs1, c2n, cb, rb0, orow, lane); break;
        case 2: recompose_row_odd<2, DEEP>(cb0, cs0, cs1, c2n, cb, rb0, orow, lane); break;
        default: recompose_row_odd<3, DEEP>(cb0, cs0, cs1, c2n, cb, rb0, orow, lane); break;
    }
}

// decode of a staged tile: two threads per 32-value block, each transposing
// one half; rows are taken in reverse tile order, so that value v's word has
// plane p at bit num - 1 - p, its negabinary digits in place
// (NegaBinaryBPEncoder.hpp:132-192); value v of block t -> cb[t * CB_LD + v].
// FAST: 2^(exp - num) is a normal float (one exact multiplication).
template <bool FAST>
__device__ __forceinline__ void decode_tile(const uint32_t* __restrict__ tile, float* __restrict__ cb, uint32_t nbk,
                                            int num, int exp, bool neg, float dscale) {
    for (uint32_t i = threadIdx.x; i < 2 * nbk; i += blockDim.x) {
        const uint32_t t = i >> 1;
        const int half = i & 1;
        float* dst = cb + t * CB_LD + 16 * half;
        // row r of the transpose is tile word 31 - r: words 4q.. (rows
        // 31-4q..28-4q) meet words 16+4q.. (rows 15-4q..12-4q) in the first
        // stage, so each pair of 16-byte reads is consumed at once
        const uint4* src = reinterpret_cast<const uint4*>(tile + t * TB_LD);
        const uint32_t sel16 = half ? 0x7632u : 0x5410u;
        uint32_t a[16];
#pragma unroll
        for (int q = 0; q < 4; q++) {
            const uint4 hi = src[q], lo = src[q + 4];
            a[15 - 4 * q] = __byte_perm(lo.x, hi.x, sel16);
            a[14 - 4 * q] = __byte_perm(lo.y, hi.y, sel16);
            a[13 - 4 * q] = __byte_perm(lo.z, hi.z, sel16);
            a[12 - 4 * q] = __byte_perm(lo.w, hi.w, sel16);
        }
        transpose32_half_tail(a);
        float f[16];
#pragma unroll
        for (int v = 0; v < 16; v++) {
            const int32_t iv = nb_to_bin(a[v]);
            if constexpr (FAST) f[v] = (float)iv * dscale;
            else f[v] = neg ? -ldexpf((float)iv, exp - num) : ldexpf((float)iv, exp - num);
        }
#pragma unroll
        for (int q = 0; q < 4; q++)
            reinterpret_cast<float4*>(dst)[q] = make_float4(f[4 * q], f[4 * q + 1], f[4 * q + 2], f[4 * q + 3]);
    }
}


__global__ void __launch_bounds__(256, 5) k_decode_recompose_nb32_odd(const uint32_t* __restrict__ base, uint64_t stride,
                                                                  const uint32_t* __restrict__ maxkey,
                                                                  const uint8_t* __restrict__ dnum,
                                                                  const float* __restrict__ coarse, Box F, Box C,
                                                                  float* __restrict__ out, uint64_t s0, uint64_t s1,
                                                                  uint32_t tld) {
    extern __shared__ __align__(16) uint32_t smem[];
    uint32_t* tiles = smem;                                  // [block][TB_LD]
    float* cb = (float*)(smem + TB_LD * tld);                // [block][CB_LD]
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int num = dnum[0];
    const int exp = frexp_exp(__uint_as_float(*maxkey)) + 2;
    const bool neg = num != 0 && (num & 1);                  // NegaBinaryBPEncoder.hpp:153, :177
    const bool dfast = (exp - num) >= -126 && (exp - num) <= 127;
    const float dscale = dfast ? (neg ? -pow2f_(exp - num) : pow2f_(exp - num)) : 1.f;
    const uint32_t rows = F.n[0] * F.n[1];
    auto block_range = [&](uint32_t r, uint64_t& fb, uint32_t& nbk) { fused_block_range(r, rows, F, C, fb, nbk); };
    // plane p of block j -> tile[j * TB_LD + 32 - num + p] (so that the
    // transposed words hold plane p at bit num - 1 - p); warp w copies planes
    // w, w+8, ..
    const int poff = 32 - num;
    auto fetch = [&](uint64_t fb, uint32_t nbk, uint32_t* tile) {
        for (int p = warp; p < num; p += 8) {
            const uint32_t* src = base + (uint64_t)p * stride + fb;
            for (uint32_t j = lane; j < nbk; j += 32) cp_async4(tile + j * TB_LD + poff + p, src + j);
        }
        cp_async_commit();
    };
    uint32_t rho0 = blockIdx.x * 8;
    if (rho0 >= rows) return;
    // block ranges of the CTA's iterations, computed by one thread two
    // iterations ahead: slot k % 3 holds iteration k's range
    __shared__ uint64_t s_fb[3];
    __shared__ uint32_t s_nbk[3];
    const uint32_t step = gridDim.x * 8;
    if (threadIdx.x == 0) {
        block_range(rho0, s_fb[0], s_nbk[0]);
        if (rho0 + step < rows) block_range(rho0 + step, s_fb[1], s_nbk[1]);
    }
    // the tile words of the planes not retrieved stay zero
    for (uint32_t i = threadIdx.x; i < tld * poff; i += blockDim.x) {
        const uint32_t row = i / poff, p = i - row * poff;
        tiles[row * TB_LD + p] = 0u;
    }
    __syncthreads();
    fetch(s_fb[0], s_nbk[0], tiles);
    for (int it = 0; rho0 < rows; it++, rho0 += step) {
        const uint32_t* tile = tiles;
        cp_async_wait_all();
        __syncthreads();
        const uint64_t fb = s_fb[it % 3];
        const uint32_t nbk = s_nbk[it % 3];
        if (threadIdx.x == 0 && rho0 + 2 * step < rows) block_range(rho0 + 2 * step, s_fb[(it + 2) % 3], s_nbk[(it + 2) % 3]);
        if (dfast) decode_tile<true>(tile, cb, nbk, num, exp, neg, dscale);
        else decode_tile<false>(tile, cb, nbk, num, exp, neg, dscale);
        __syncthreads();
        // the tile is free again: fetch the next rows' planes during the recomposition
        if (rho0 + step < rows) fetch(s_fb[(it + 1) % 3], s_nbk[(it + 1) % 3], tiles);
        const uint32_t rho = rho0 + warp;
        if (rho < rows) recompose_fine_row(fused_row(rho, F, C, s0, s1, fb), C, coarse, out, cb, lane);
    }
    cp_async_wait_all();
}

// The finest levels of many fields in one persistent launch (the batched
// retrieval): the global 8-row units of all segments are walked as in
// k_decode_recompose_nb32_odd, with each unit's field looked up in the segment
// table (one segment per field, odd row lengths). The plane count, exponent
// and decode scale are the unit's field's; a fetch zeroes the tile words of
// the planes its field did not retrieve. Staging, decode and recomposition
// are those of the single-field kernel, so the results are bit-identical.
__global__ void __launch_bounds__(256, 4) k_decode_recompose_nb32_multi(const FusedSeg* __restrict__ segs, int nseg,
                                                                       uint64_t total, uint32_t tld) {
    extern __shared__ __align__(16) uint32_t smem[];
    uint32_t* tiles = smem;                                  // [block][TB_LD]
    float* cb = (float*)(smem + TB_LD * tld);                // [block][CB_LD]
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    __shared__ int s_seg[3];
    __shared__ uint64_t s_fb[3];
    __shared__ uint32_t s_nbk[3];
    const uint64_t step = gridDim.x;
    uint64_t u = blockIdx.x;
    if (u >= total) return;
    // thread 0: the field and block range of unit g into slot k
    auto plan = [&](uint64_t g, int k) {
        const int s = find_seg(segs, nseg, g, &FusedSeg::unit_begin);
        const FusedSeg& q = segs[s];
        s_seg[k] = s;
        fused_block_range((uint32_t)(g - q.unit_begin) * 8, q.F.n[0] * q.F.n[1], q.F, q.C, s_fb[k], s_nbk[k]);
    };
    auto fetch = [&](int k) {
        const FusedSeg& q = segs[s_seg[k]];
        const int num = *q.dnum;
        const int poff = 32 - num;
        const uint64_t fb = s_fb[k];
        const uint32_t nbk = s_nbk[k];
        for (uint32_t i = threadIdx.x; i < nbk * (uint32_t)poff; i += blockDim.x) {
            const uint32_t row = i / poff, p = i - row * poff;
            tiles[row * TB_LD + p] = 0u;
        }
        for (int p = warp; p < num; p += 8) {
            const uint32_t* src = q.base + (uint64_t)p * q.stride + fb;
            for (uint32_t j = lane; j < nbk; j += 32) cp_async4(tiles + j * TB_LD + poff + p, src + j);
        }
        cp_async_commit();
    };
    if (threadIdx.x == 0) {
        plan(u, 0);
        if (u + step < total) plan(u + step, 1);
    }
    __syncthreads();
    fetch(0);
    for (int it = 0; u < total; it++, u += step) {
        cp_async_wait_all();
        __syncthreads();
        const int k = it % 3;
        const FusedSeg& q = segs[s_seg[k]];
        const uint64_t fb = s_fb[k];
        const uint32_t nbk = s_nbk[k];
        if (threadIdx.x == 0 && u + 2 * step < total) plan(u + 2 * step, (it + 2) % 3);
        const int num = *q.dnum;
        const int exp = frexp_exp(__uint_as_float(*q.key)) + 2;
        const bool neg = num != 0 && (num & 1);              // NegaBinaryBPEncoder.hpp:153, :177
        const bool dfast = (exp - num) >= -126 && (exp - num) <= 127;
        const float dscale = dfast ? (neg ? -pow2f_(exp - num) : pow2f_(exp - num)) : 1.f;
        if (dfast) decode_tile<true>(tiles, cb, nbk, num, exp, neg, dscale);
        else decode_tile<false>(tiles, cb, nbk, num, exp, neg, dscale);
        __syncthreads();
        // the tile is free again: fetch the next unit's planes during the recomposition
        if (u + step < total) fetch((it + 1) % 3);
        const uint32_t rows = q.F.n[0] * q.F.n[1];
        const uint32_t rho = (uint32_t)(u - q.unit_begin) * 8 + warp;
        if (rho < rows) recompose_fine_row(fused_row(rho, q.F, q.C, q.s0, q.s1, fb), q.C, q.coarse, q.out, cb, lane);
    }
    cp_async_wait_all();
}

// decode of a plane-major tile (row 32 - num + p = plane p, rows below zero;
// block t of the range at column t): the same half transposes, each thread
// reading its block's 32 rows and combining rows 31-k and 15-k at once
template <bool FAST, int RS>
__device__ __forceinline__ void decode_tile_pm(const uint32_t* __restrict__ tile, float* __restrict__ cb,
                                               uint32_t nbk, int num, int exp, bool neg, float dscale,
                                               uint32_t tid = threadIdx.x, uint32_t nthreads = blockDim.x) {
    for (uint32_t i = tid; i < 2 * nbk; i += nthreads) {
        const uint32_t t = i >> 1;
        const int half = i & 1;
        float* dst = cb + t * CB_LD + 16 * half;
        const uint32_t* col = tile + t;
        const uint32_t sel16 = half ? 0x7632u : 0x5410u;
        uint32_t a[16];
#pragma unroll
        for (int k = 0; k < 16; k++) a[k] = __byte_perm(col[(31 - k) * RS], col[(15 - k) * RS], sel16);
        transpose32_half_tail(a);
        float f[16];
#pragma unroll
        for (int v = 0; v < 16; v++) {
            const int32_t iv = nb_to_bin(a[v]);
            if constexpr (FAST) f[v] = (float)iv * dscale;
            else f[v] = neg ? -ldexpf((float)iv, exp - num) : ldexpf((float)iv, exp - num);
        }
#pragma unroll
        for (int q = 0; q < 4; q++)
            reinterpret_cast<float4*>(dst)[q] = make_float4(f[4 * q], f[4 * q + 1], f[4 * q + 2], f[4 * q + 3]);
    }
}

// Odd row length, planes staged by TMA: per CTA iteration (8 rows) one
// elected warp issues one 2-D tensor copy per retrieved plane (box: `bw`
// words of that plane's row, from the 16-byte aligned block fb & ~3) into the
// plane-major tile, completing on an mbarrier; the copy for the next
// iteration is issued once the tile is decoded and overlaps the
// recomposition. Every wait on the mbarrier is bounded by `wait_limit` SM
// cycles: a CTA whose wait gives up writes PRODM_ETIMEOUT to *status, waits
// (bounded again) for its copies in flight and returns. `tx_extra` raises the
// expected byte count (0 in normal use; a positive value makes every wait run
// out, which is how the timeout path is tested).
template <int RS>
__global__ void __launch_bounds__(256, 5) k_decode_recompose_nb32_tma(
    const __grid_constant__ CUtensorMap tmap, uint32_t bw, const uint32_t* __restrict__ maxkey,
    const uint8_t* __restrict__ dnum, const float* __restrict__ coarse, Box F, Box C, float* __restrict__ out,
    uint64_t s0, uint64_t s1, int* __restrict__ status, long long wait_limit, uint32_t tx_extra, int tall) {
    extern __shared__ __align__(128) uint32_t tma_smem[];
    uint32_t* tile = tma_smem;                               // [32][RS] plane-major
    float* cb = (float*)(tma_smem + 32 * RS);                // [block][CB_LD]
    __shared__ __align__(8) uint64_t bar;
    __shared__ uint64_t s_fb[3];
    __shared__ uint32_t s_nbk[3];
    __shared__ FusedRow s_row[2][8];   // the rows of iterations it (slot it & 1) and it + 1
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int num = dnum[0];
    const int exp = frexp_exp(__uint_as_float(*maxkey)) + 2;
    const bool neg = num != 0 && (num & 1);                  // NegaBinaryBPEncoder.hpp:153, :177
    const bool dfast = (exp - num) >= -126 && (exp - num) <= 127;
    const float dscale = dfast ? (neg ? -pow2f_(exp - num) : pow2f_(exp - num)) : 1.f;
    const uint32_t rows = F.n[0] * F.n[1];
    const int poff = 32 - num;
    // lanes 0..7 of warp 0: the rows of the iteration starting at r, block range fb
    auto rows_of = [&](uint32_t r, uint64_t fb, FusedRow* slot) {
        if (lane < 8 && r + lane < rows) slot[lane] = fused_row(r + lane, F, C, s0, s1, fb);
    };
    uint32_t rho0 = blockIdx.x * 8;
    if (rho0 >= rows) return;
    if ((smem_addr(tile) & 127u) != 0) {   // TMA destinations need 128-byte alignment
        if (threadIdx.x == 0) atomicExch(status, PRODM_ECUDA);
        return;
    }
    const uint32_t step = gridDim.x * 8;
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        fused_block_range(rho0, rows, F, C, s_fb[0], s_nbk[0]);
        if (rho0 + step < rows) fused_block_range(rho0 + step, rows, F, C, s_fb[1], s_nbk[1]);
    }
    if (!tall)
        for (uint32_t i = threadIdx.x; i < (uint32_t)poff * RS; i += blockDim.x) tile[i] = 0u;   // planes not retrieved
    __syncthreads();
    if (warp == 0) rows_of(rho0, s_fb[0], s_row[0]);
    const uint32_t bytes = (tall ? 32u * RS : (uint32_t)num * bw) * 4u + tx_extra;
    auto issue = [&](uint64_t fb) {   // warp 0
        if (lane == 0) mbar_arrive_expect_tx(&bar, bytes);
        __syncwarp();
        const int x = (int)(fb & ~3ull);
        if (tall) {   // one box of all 32 tile rows; rows of planes below 0 arrive as zeros
            if (lane == 0) tma_load_2d(tile, &tmap, x, num - 32, &bar);
        } else {
            for (int p = lane; p < num; p += 32) tma_load_2d(tile + (poff + p) * RS, &tmap, x, p, &bar);
        }
    };
    if (warp == 0) issue(s_fb[0]);
    // the first tile is on its way; the coarse box and the output belong to
    // the previous launches (the plane counts and the planes are older)
    pdl_wait();
    pdl_release();
    uint32_t parity = 0;
    for (int it = 0; rho0 < rows; it++, rho0 += step) {
        const bool ok = mbar_wait_bounded(&bar, parity, wait_limit);
        if (__syncthreads_or(!ok)) {
            if (threadIdx.x == 0) atomicExch(status, PRODM_ETIMEOUT);
            mbar_wait_bounded(&bar, parity, wait_limit);
            return;
        }
        parity ^= 1u;
        const uint64_t fb = s_fb[it % 3];
        const uint32_t nbk = s_nbk[it % 3];
        if (threadIdx.x == 0 && rho0 + 2 * step < rows)
            fused_block_range(rho0 + 2 * step, rows, F, C, s_fb[(it + 2) % 3], s_nbk[(it + 2) % 3]);
        const uint32_t* t0 = tile + (fb & 3u);
        if (dfast) decode_tile_pm<true, RS>(t0, cb, nbk, num, exp, neg, dscale);
        else decode_tile_pm<false, RS>(t0, cb, nbk, num, exp, neg, dscale);
        __syncthreads();
        // the tile is free again: the next rows' planes arrive during the recomposition
        if (warp == 0 && rho0 + step < rows) {
            fence_proxy_async_smem();
            issue(s_fb[(it + 1) % 3]);
            rows_of(rho0 + step, s_fb[(it + 1) % 3], s_row[(it + 1) & 1]);
        }
        if (rho0 + warp < rows) recompose_fine_row(s_row[it & 1][warp], C, coarse, out, cb, lane);
    }
}

// The TMA kernel over the finest levels of many fields (the batched
// retrieval): each field's planes have their own tensor map in device memory
// (FusedSeg::map, written before the launch; box FusedSeg::bw words <= RS),
// each unit's field is looked up in the segment table. A unit is
// FusedSeg::rpu consecutive rows (8 per warp-round; short rows take several
// rounds, so that a unit moves about as many values as 8 rows of 257). Tile rows below a
// unit's planes must be zero; the copies write rows 32 - num .. 31, so rows
// below the lowest row copied so far are zero, and only a unit with fewer
// planes than that zeroes the rows in between before its copies are issued.
// Decode, recomposition and the bounded waits are those of
// k_decode_recompose_nb32_tma, so results are bit-identical.
template <int RS>
__global__ void __launch_bounds__(256, 5) k_decode_recompose_nb32_tma_multi(const FusedSeg* __restrict__ segs, int nseg,
                                                                           uint64_t total, int* __restrict__ status,
                                                                           long long wait_limit, uint32_t tx_extra) {
    extern __shared__ __align__(128) uint32_t tma_smem[];
    uint32_t* tile = tma_smem;                               // [32][RS] plane-major
    float* cb = (float*)(tma_smem + 32 * RS);                // [block][CB_LD]
    __shared__ __align__(8) uint64_t bar;
    __shared__ int s_seg[3];
    __shared__ uint64_t s_fb[3];
    __shared__ uint32_t s_nbk[3];
    __shared__ FusedRow s_row[2][kMaxUnitRows];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint64_t step = gridDim.x;
    uint64_t u = blockIdx.x;
    if (u >= total) return;
    if ((smem_addr(tile) & 127u) != 0) {   // TMA destinations need 128-byte alignment
        if (threadIdx.x == 0) atomicExch(status, PRODM_ECUDA);
        return;
    }
    // thread 0: the field and block range of unit g into slot k
    auto plan = [&](uint64_t g, int k) {
        const int s = find_seg(segs, nseg, g, &FusedSeg::unit_begin);
        const FusedSeg& q = segs[s];
        s_seg[k] = s;
        fused_block_range((uint32_t)(g - q.unit_begin) * q.rpu, q.F.n[0] * q.F.n[1], q.F, q.C, s_fb[k], s_nbk[k],
                          q.rpu);
    };
    // every thread: rows [zlo, 32 - num) zeroed for the unit in slot k (rows
    // below zlo are zero already; a tall copy writes zeros there itself);
    // afterwards rows below 32 - num are zero
    uint32_t zlo = 0;
    auto zero_rows = [&](int k) {
        const FusedSeg& q = segs[s_seg[k]];
        const uint32_t lo = 32u - *q.dnum;
        if (!q.tall)
            for (uint32_t i = zlo * RS + threadIdx.x; i < lo * RS; i += blockDim.x) tile[i] = 0u;
        zlo = lo;
    };
    // warp 0: the copies of the unit in slot k, and the row geometry of unit g
    auto issue = [&](int k, uint64_t g, FusedRow* rows) {
        const FusedSeg& q = segs[s_seg[k]];
        const int num = *q.dnum;
        if (lane == 0) mbar_arrive_expect_tx(&bar, (q.tall ? 32u * RS : (uint32_t)num * q.bw) * 4u + tx_extra);
        __syncwarp();
        const int x = (int)(s_fb[k] & ~3ull);
        if (q.tall) {   // one box of all 32 tile rows; rows of planes below 0 arrive as zeros
            if (lane == 0) tma_load_2d(tile, (const CUtensorMap*)q.map, x, num - 32, &bar);
        } else {
            for (int p = lane; p < num; p += 32)
                tma_load_2d(tile + (32 - num + p) * RS, (const CUtensorMap*)q.map, x, p, &bar);
        }
        const uint32_t r0 = (uint32_t)(g - q.unit_begin) * q.rpu, nr = q.F.n[0] * q.F.n[1];
        for (uint32_t r = lane; r < q.rpu; r += 32)
            if (r0 + r < nr) rows[r] = fused_row(r0 + r, q.F, q.C, q.s0, q.s1, s_fb[k]);
    };
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        plan(u, 0);
        if (u + step < total) plan(u + step, 1);
    }
    __syncthreads();
    zero_rows(0);
    __syncthreads();
    if (warp == 0) issue(0, u, s_row[0]);
    uint32_t parity = 0;
    for (int it = 0; u < total; it++, u += step) {
        const bool ok = mbar_wait_bounded(&bar, parity, wait_limit);
        if (__syncthreads_or(!ok)) {
            if (threadIdx.x == 0) atomicExch(status, PRODM_ETIMEOUT);
            mbar_wait_bounded(&bar, parity, wait_limit);
            return;
        }
        parity ^= 1u;
        const int k = it % 3;
        const FusedSeg& q = segs[s_seg[k]];
        const uint64_t fb = s_fb[k];
        const uint32_t nbk = s_nbk[k];
        if (threadIdx.x == 0 && u + 2 * step < total) plan(u + 2 * step, (it + 2) % 3);
        const int num = *q.dnum;
        const int exp = frexp_exp(__uint_as_float(*q.key)) + 2;
        const bool neg = num != 0 && (num & 1);              // NegaBinaryBPEncoder.hpp:153, :177
        const bool dfast = (exp - num) >= -126 && (exp - num) <= 127;
        const float dscale = dfast ? (neg ? -pow2f_(exp - num) : pow2f_(exp - num)) : 1.f;
        const uint32_t* t0 = tile + (fb & 3u);
        if (dfast) decode_tile_pm<true, RS>(t0, cb, nbk, num, exp, neg, dscale);
        else decode_tile_pm<false, RS>(t0, cb, nbk, num, exp, neg, dscale);
        __syncthreads();
        // the tile is free again: the next unit's rows below its planes are
        // zeroed (rows the copies do not write) and its planes arrive during
        // the recomposition
        if (u + step < total) {
            zero_rows((it + 1) % 3);
            if (warp == 0) {
                fence_proxy_async_smem();
                issue((it + 1) % 3, u + step, s_row[(it + 1) & 1]);
            }
        }
        const uint32_t rows = q.F.n[0] * q.F.n[1];
        const uint32_t rho0 = (uint32_t)(u - q.unit_begin) * q.rpu;
        for (uint32_t r = warp; r < q.rpu && rho0 + r < rows; r += 8)
            recompose_fine_row(s_row[it & 1][r], q.C, q.coarse, q.out, cb, lane);
    }
}

// Warp-specialised form of the TMA kernel: 16 warps, warps 0..ND-1 decode and
// the other 16 - ND recompose (a unit is 16 - ND consecutive rows, one per
// recomposition warp), with both the plane tile and the coefficient tile
// double buffered, so the decode of unit it + 1 runs while unit it is
// recomposed. The groups meet only on mbarriers: tile_full (the TMA bytes of
// a unit's planes), coef_full (all decode threads arrived after writing a
// unit's coefficients and row geometry) and coef_empty (all recomposition
// threads arrived after their rows). The decode warps stay in step with a
// named barrier; with 64 registers the recomposition keeps six column groups
// in flight (four for four-corner rows). Every wait is bounded by
// `wait_limit` SM cycles. A decode thread whose wait gives up raises a
// shared flag that the whole decode group reads after its barrier (so the
// group leaves together: it writes PRODM_ETIMEOUT to *status, lets its copies
// in flight land, bounded again, and returns); a recomposition warp that
// gives up writes the status and returns, and the other group's waits then
// run out too.
template <int RS, int ND>
__global__ void __launch_bounds__(512, 2) k_decode_recompose_nb32_ws(
    const __grid_constant__ CUtensorMap tmap, uint32_t bw, const uint32_t* __restrict__ maxkey,
    const uint8_t* __restrict__ dnum, const float* __restrict__ coarse, Box F, Box C, float* __restrict__ out,
    uint64_t s0, uint64_t s1, uint32_t tld, int* __restrict__ status, long long wait_limit, uint32_t tx_extra,
    int tall) {
    extern __shared__ __align__(128) uint32_t ws_smem[];
    uint32_t* tiles = ws_smem;                               // [2][32][RS] plane-major
    float* cbs = (float*)(ws_smem + 2 * 32 * RS);            // [2][tld][CB_LD]
    __shared__ __align__(8) uint64_t bar_tile[2], bar_full[2], bar_empty[2];
    __shared__ uint64_t s_fb[2];
    __shared__ uint32_t s_nbk[2];
    constexpr int NR = 16 - ND;                              // recomposition warps = rows per unit
    __shared__ FusedRow s_row[2][NR];
    __shared__ volatile int s_abort;
    constexpr int GROUP = 32 * ND, RGROUP = 32 * NR;         // threads of the decode / recomposition group
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const bool dec = threadIdx.x < GROUP;
    const int num = dnum[0];
    const int exp = frexp_exp(__uint_as_float(*maxkey)) + 2;
    const bool neg = num != 0 && (num & 1);                  // NegaBinaryBPEncoder.hpp:153, :177
    const bool dfast = (exp - num) >= -126 && (exp - num) <= 127;
    const float dscale = dfast ? (neg ? -pow2f_(exp - num) : pow2f_(exp - num)) : 1.f;
    const uint32_t rows = F.n[0] * F.n[1];
    const uint32_t nunits = (rows + NR - 1) / NR;
    const int poff = 32 - num;
    const uint32_t u0 = blockIdx.x, step = gridDim.x;
    if (u0 >= nunits) return;
    const int myunits = (int)((nunits - u0 + step - 1) / step);
    if ((smem_addr(tiles) & 127u) != 0) {   // TMA destinations need 128-byte alignment
        if (threadIdx.x == 0) atomicExch(status, PRODM_ECUDA);
        return;
    }
    if (threadIdx.x == 0) {
        s_abort = 0;
        mbar_init(&bar_tile[0], 1);
        mbar_init(&bar_tile[1], 1);
        mbar_init(&bar_full[0], GROUP);
        mbar_init(&bar_full[1], GROUP);
        mbar_init(&bar_empty[0], RGROUP);
        mbar_init(&bar_empty[1], RGROUP);
    }
    if (!tall)
        for (uint32_t i = threadIdx.x; i < (uint32_t)poff * RS; i += blockDim.x) {   // planes not retrieved
            tiles[i] = 0u;
            tiles[32 * RS + i] = 0u;
        }
    __syncthreads();
    const uint32_t bytes = (tall ? 32u * RS : (uint32_t)num * bw) * 4u + tx_extra;
    // warp 0: block range of unit k of this CTA into slot b, then its planes into tile b
    auto issue = [&](int k, int b) {
        if (lane == 0) {
            const uint32_t r0 = (u0 + (uint32_t)k * step) * NR;
            fused_block_range(r0, rows, F, C, s_fb[b], s_nbk[b], NR);
            mbar_arrive_expect_tx(&bar_tile[b], bytes);
        }
        __syncwarp();
        const int x = (int)(s_fb[b] & ~3ull);
        uint32_t* tile = tiles + b * 32 * RS;
        if (tall) {   // one box of all 32 tile rows; rows of planes below 0 arrive as zeros
            if (lane == 0) tma_load_2d(tile, &tmap, x, num - 32, &bar_tile[b]);
        } else {
            for (int p = lane; p < num; p += 32) tma_load_2d(tile + (poff + p) * RS, &tmap, x, p, &bar_tile[b]);
        }
    };
    if (warp == 0) {
        issue(0, 0);
        if (myunits > 1) issue(1, 1);
    }
    // the first tiles are on their way; the coarse box and the output belong
    // to the previous launches (the plane counts and the planes are older)
    pdl_wait();
    pdl_release();
    if (dec) {
        for (int it = 0; it < myunits; it++) {
            const int b = it & 1;
            const uint32_t ph = (uint32_t)(it >> 1) & 1u;
            bool ok = mbar_wait_bounded(&bar_tile[b], ph, wait_limit);
            ok = ok && mbar_wait_bounded(&bar_empty[b], ph ^ 1u, wait_limit);   // first use: the phase before is done
            if (!ok) s_abort = 1;   // read by the whole group after its next barrier
            const uint64_t fb = s_fb[b];
            const uint32_t nbk = s_nbk[b];
            if (warp == 0 && lane < NR) {
                const uint32_t r = (u0 + (uint32_t)it * step) * NR + lane;
                if (r < rows) s_row[b][lane] = fused_row(r, F, C, s0, s1, fb);
                else s_row[b][lane].m01 = -1;
            }
            const uint32_t* t0 = tiles + b * 32 * RS + (fb & 3u);
            float* cb = cbs + (size_t)b * tld * CB_LD;
            if (dfast) decode_tile_pm<true, RS>(t0, cb, nbk, num, exp, neg, dscale, threadIdx.x, GROUP);
            else decode_tile_pm<false, RS>(t0, cb, nbk, num, exp, neg, dscale, threadIdx.x, GROUP);
            mbar_arrive(&bar_full[b]);
            group_sync(GROUP);   // tile b is decoded: it may take unit it + 2
            if (s_abort) {   // a wait gave up: report, let the copies in flight land, leave
                if (threadIdx.x == 0) atomicExch(status, PRODM_ETIMEOUT);
                mbar_wait_bounded(&bar_tile[b], ph, wait_limit);
                if (it + 1 < myunits) mbar_wait_bounded(&bar_tile[b ^ 1], ((uint32_t)(it + 1) >> 1) & 1u, wait_limit);
                return;
            }
            if (warp == 0 && it + 2 < myunits) {
                fence_proxy_async_smem();
                issue(it + 2, b);
            }
        }
    } else {
        const int rw = warp - GROUP / 32;
        for (int it = 0; it < myunits; it++) {
            const int b = it & 1;
            const uint32_t ph = (uint32_t)(it >> 1) & 1u;
            if (!mbar_wait_bounded(&bar_full[b], ph, wait_limit)) {
                if (lane == 0) atomicExch(status, PRODM_ETIMEOUT);
                return;
            }
            const FusedRow r = s_row[b][rw];
            if (r.m01 >= 0) recompose_fine_row<true>(r, C, coarse, out, cbs + (size_t)b * tld * CB_LD, lane);
            mbar_arrive(&bar_empty[b]);
        }
    }
}

// The warp-specialised kernel over the finest levels of many fields (the
// batched retrieval): units of 16 - ND rows of one field, found in the
// segment table as in k_decode_recompose_nb32_tma_multi; every field's
// tensor map is a tall one (box of RS words x 32 plane rows), so the tiles
// are never zeroed and the plane count may change from unit to unit. The
// field of the unit in tile b is kept for the recomposition group in
// s_rseg[b] (written with the unit's row geometry, before coef_full).
// Decode, recomposition and the bounded waits are those of
// k_decode_recompose_nb32_ws, so results are bit-identical.
template <int RS, int ND>
__global__ void __launch_bounds__(512, 2) k_decode_recompose_nb32_ws_multi(const FusedSeg* __restrict__ segs, int nseg,
                                                                          uint64_t total, uint32_t tld,
                                                                          int* __restrict__ status,
                                                                          long long wait_limit, uint32_t tx_extra) {
    extern __shared__ __align__(128) uint32_t ws_smem[];
    uint32_t* tiles = ws_smem;                               // [2][32][RS] plane-major
    float* cbs = (float*)(ws_smem + 2 * 32 * RS);            // [2][tld][CB_LD]
    constexpr int NR = 16 - ND;
    constexpr int GROUP = 32 * ND, RGROUP = 32 * NR;
    __shared__ __align__(8) uint64_t bar_tile[2], bar_full[2], bar_empty[2];
    __shared__ uint64_t s_fb[2];
    __shared__ uint32_t s_nbk[2];
    __shared__ int s_seg[2], s_rseg[2];
    __shared__ FusedRow s_row[2][NR];
    __shared__ volatile int s_abort;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const bool dec = threadIdx.x < GROUP;
    const uint64_t u0 = blockIdx.x, step = gridDim.x;
    if (u0 >= total) return;
    const int myunits = (int)((total - u0 + step - 1) / step);
    if ((smem_addr(tiles) & 127u) != 0) {   // TMA destinations need 128-byte alignment
        if (threadIdx.x == 0) atomicExch(status, PRODM_ECUDA);
        return;
    }
    if (threadIdx.x == 0) {
        s_abort = 0;
        mbar_init(&bar_tile[0], 1);
        mbar_init(&bar_tile[1], 1);
        mbar_init(&bar_full[0], GROUP);
        mbar_init(&bar_full[1], GROUP);
        mbar_init(&bar_empty[0], RGROUP);
        mbar_init(&bar_empty[1], RGROUP);
    }
    __syncthreads();
    // lane 0 of warp 0: field and block range of unit k of this CTA into slot b, its planes into tile b
    auto issue = [&](int k, int b) {
        if (lane == 0) {
            const uint64_t g = u0 + (uint64_t)k * step;
            const int sg = find_seg(segs, nseg, g, &FusedSeg::unit_begin);
            const FusedSeg& q = segs[sg];
            s_seg[b] = sg;
            fused_block_range((uint32_t)(g - q.unit_begin) * NR, q.F.n[0] * q.F.n[1], q.F, q.C, s_fb[b], s_nbk[b], NR);
            mbar_arrive_expect_tx(&bar_tile[b], 32u * RS * 4u + tx_extra);
            // one box of all 32 tile rows; rows of planes below 0 arrive as zeros
            tma_load_2d(tiles + b * 32 * RS, (const CUtensorMap*)q.map, (int)(s_fb[b] & ~3ull), (int)*q.dnum - 32,
                        &bar_tile[b]);
        }
    };
    if (warp == 0) {
        issue(0, 0);
        if (myunits > 1) issue(1, 1);
    }
    // the first tiles are on their way; the coarse boxes and the outputs belong
    // to the previous launches (the plane counts and the planes are older)
    pdl_wait();
    pdl_release();
    if (dec) {
        for (int it = 0; it < myunits; it++) {
            const int b = it & 1;
            const uint32_t ph = (uint32_t)(it >> 1) & 1u;
            bool ok = mbar_wait_bounded(&bar_tile[b], ph, wait_limit);
            ok = ok && mbar_wait_bounded(&bar_empty[b], ph ^ 1u, wait_limit);   // first use: the phase before is done
            if (!ok) s_abort = 1;   // read by the whole group after its next barrier
            const int sg = s_seg[b];
            const FusedSeg& q = segs[sg];
            const uint64_t fb = s_fb[b];
            const uint32_t nbk = s_nbk[b];
            if (warp == 0 && lane < NR) {
                const uint64_t g = u0 + (uint64_t)it * step;
                const uint32_t r = (uint32_t)(g - q.unit_begin) * NR + lane;
                if (r < q.F.n[0] * q.F.n[1]) s_row[b][lane] = fused_row(r, q.F, q.C, q.s0, q.s1, fb);
                else s_row[b][lane].m01 = -1;
                if (lane == 0) s_rseg[b] = sg;
            }
            const int num = *q.dnum;
            const int exp = frexp_exp(__uint_as_float(*q.key)) + 2;
            const bool neg = num != 0 && (num & 1);          // NegaBinaryBPEncoder.hpp:153, :177
            const bool dfast = (exp - num) >= -126 && (exp - num) <= 127;
            const float dscale = dfast ? (neg ? -pow2f_(exp - num) : pow2f_(exp - num)) : 1.f;
            const uint32_t* t0 = tiles + b * 32 * RS + (fb & 3u);
            float* cb = cbs + (size_t)b * tld * CB_LD;
            if (dfast) decode_tile_pm<true, RS>(t0, cb, nbk, num, exp, neg, dscale, threadIdx.x, GROUP);
            else decode_tile_pm<false, RS>(t0, cb, nbk, num, exp, neg, dscale, threadIdx.x, GROUP);
            mbar_arrive(&bar_full[b]);
            group_sync(GROUP);   // tile b is decoded: it may take unit it + 2
            if (s_abort) {   // a wait gave up: report, let the copies in flight land, leave
                if (threadIdx.x == 0) atomicExch(status, PRODM_ETIMEOUT);
                mbar_wait_bounded(&bar_tile[b], ph, wait_limit);
                if (it + 1 < myunits) mbar_wait_bounded(&bar_tile[b ^ 1], ((uint32_t)(it + 1) >> 1) & 1u, wait_limit);
                return;
            }
            if (warp == 0 && it + 2 < myunits) {
                fence_proxy_async_smem();
                issue(it + 2, b);
            }
        }
    } else {
        const int rw = warp - ND;
        for (int it = 0; it < myunits; it++) {
            const int b = it & 1;
            const uint32_t ph = (uint32_t)(it >> 1) & 1u;
            if (!mbar_wait_bounded(&bar_full[b], ph, wait_limit)) {
                if (lane == 0) atomicExch(status, PRODM_ETIMEOUT);
                return;
            }
            const FusedRow r = s_row[b][rw];
            const FusedSeg& q = segs[s_rseg[b]];
            if (r.m01 >= 0) recompose_fine_row<true>(r, q.C, q.coarse, q.out, cbs + (size_t)b * tld * CB_LD, lane);
            mbar_arrive(&bar_empty[b]);
        }
    }
}

}  // namespace

static uint32_t fused_max_blocks(const Box& F) { return (8 * F.n[2] + 31) / 32 + 2; }
static size_t fused_smem(const Box& F) {
    const uint32_t mb = fused_max_blocks(F);
    if (F.n[2] & 1u) return (size_t)mb * TB_LD * 4 + (size_t)mb * CB_LD * 4;
    return (size_t)mb * 32 * 4 + (size_t)(mb | 1u) * 32 * 4;
}

bool decode_recompose_nb32_ok(const Box& F) {
    const uint64_t rows = (uint64_t)F.n[0] * F.n[1];
    return rows >= 1024 && fused_smem(F) <= 200 * 1024;
}

// cuTensorMapEncodeTiled through the runtime's driver entry point (no link
// against the CUDA driver library); NULL when the CUDA driver does not provide it
static PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (PFN_cuTensorMapEncodeTiled_v12000)p;
    });
    return fn;
}

static int g_tma_tx_extra = 0;                 // test hook: extra expected bytes per tile
static long long g_tma_wait_cycles = 4000000000ll;   // about two seconds at 2 GHz

void fused_tma_test_hook(int tx_extra, long long wait_cycles) {
    g_tma_tx_extra = tx_extra > 0 ? tx_extra : 0;
    g_tma_wait_cycles = wait_cycles > 0 ? wait_cycles : 4000000000ll;
}

// The TMA kernel for odd rows whose 8-row block range fits one box (at most
// 256 words): box width and tile row stride (a multiple of 32 words, so that
// every tile row starts on a 128-byte boundary).
// Which TMA kernel a fused level takes: the warp-specialised form, with
// 16 - nd rows per unit for rows of 257 values and up while its tile rows fit
// 192 words, and with 8-row units where the 8-row tile rows are 160 words or
// more; the 8-warp form below that. With 8 decode warps (before the units
// grew) the split measured at 513^3: step 3.047 ms with the 8-warp form
// everywhere, 3.008 ms warp-specialised everywhere, 2.966 ms mixed.
// PRODM_FUSED_WS overrides: 0 never, 1 always, 2 the default rule.
static int fused_ws() {
    static const int mode = [] {
        const char* v = getenv("PRODM_FUSED_WS");
        return v ? atoi(v) : 2;
    }();
    return mode;
}

// rows per unit of the warp-specialised kernel with nd decode warps (one per recomposition warp)
static uint32_t ws_unit_rows(int nd) { return 16u - (uint32_t)nd; }
static uint32_t ws_tile_blocks(const Box& F, int nd) { return (ws_unit_rows(nd) * F.n[2] + 31) / 32 + 2; }
// Decode warps of the warp-specialised kernel (the other 16 - nd warps
// recompose, one unit row each). Measured at 513^3 (level 7, CUDA events):
// 8 decode warps (8-row units) 263 us, 7: 245 us, 6: 237 us, 5: 237 us
// (step 2.692 / 2.590 / 2.543 / 2.534 ms): the recomposition group was the
// slower one. PRODM_WS_ND overrides: 5 (default), 6 or 8.
static int ws_decode_warps() {
    const char* v = getenv("PRODM_WS_ND");
    const int n = v ? atoi(v) : 5;
    return n == 6 ? 6 : (n == 8 ? 8 : 5);
}

template <int RS, int ND>
static int launch_fused_ws(const CUtensorMap& map, uint32_t bw, const void* maxkey, const uint8_t* dnum,
                           const float* coarse, const Box& F, const Box& C, float* out, uint64_t s0, uint64_t s1,
                           int* status, cudaStream_t st, bool pdl, int tall) {
    const uint32_t tld = ws_tile_blocks(F, ND), nr = ws_unit_rows(ND);
    const size_t smem = (size_t)2 * 32 * RS * 4 + (size_t)2 * tld * CB_LD * 4;
    const void* kern = (const void*)k_decode_recompose_nb32_ws<RS, ND>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return cuda_status(e, "cudaFuncSetAttribute");
    const uint64_t need = ((uint64_t)F.n[0] * F.n[1] + nr - 1) / nr;
    const unsigned grid = persistent_grid_for(kern, 512, smem, need, need);
    count_launch();
    e = launch_chain(pdl, k_decode_recompose_nb32_ws<RS, ND>, dim3(grid), dim3(512), smem, st, map, bw,
                     (const uint32_t*)maxkey, dnum, coarse, F, C, out, s0, s1, tld, status, g_tma_wait_cycles,
                     (uint32_t)g_tma_tx_extra, tall);
    if (e != cudaSuccess) return cuda_status(e, "k_decode_recompose_nb32_ws");
    return PRODM_OK;
}

template <int RS>
static int launch_fused_tma(const CUtensorMap& map, uint32_t bw, const void* maxkey, const uint8_t* dnum,
                            const float* coarse, const Box& F, const Box& C, float* out, uint64_t s0, uint64_t s1,
                            int* status, cudaStream_t st, bool pdl, int tall) {
    if (fused_ws() == 1 || (fused_ws() == 2 && RS >= 160))
        return launch_fused_ws<RS, 8>(map, bw, maxkey, dnum, coarse, F, C, out, s0, s1, status, st, pdl, tall);
    const size_t smem = (size_t)32 * RS * 4 + (size_t)fused_max_blocks(F) * CB_LD * 4;
    const void* kern = (const void*)k_decode_recompose_nb32_tma<RS>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return cuda_status(e, "cudaFuncSetAttribute");
    const uint64_t rows = (uint64_t)F.n[0] * F.n[1];
    const uint64_t need = (rows + 7) / 8;
    const unsigned grid = persistent_grid_for(kern, 256, smem, need, need);
    count_launch();
    e = launch_chain(pdl, k_decode_recompose_nb32_tma<RS>, dim3(grid), dim3(256), smem, st, map, bw,
                     (const uint32_t*)maxkey, dnum, coarse, F, C, out, s0, s1, status, g_tma_wait_cycles,
                     (uint32_t)g_tma_tx_extra, tall);
    if (e != cudaSuccess) return cuda_status(e, "k_decode_recompose_nb32_tma");
    return PRODM_OK;
}

// PRODM_TMA_TALL: 1 (default) stages a unit's planes by one tall box, 0 by one box per plane
static int tma_tall() {
    const char* v = getenv("PRODM_TMA_TALL");
    return v ? atoi(v) : 1;
}
bool fused_tma_tall() { return tma_tall() != 0; }
uint32_t fused_tma_stride(uint32_t bw) { return bw <= 96 ? 96u : (bw <= 160 ? 160u : 256u); }

// Returns PRODM_EUNSUPPORTED when the shape does not suit the row mapping
// (the caller then runs the unfused kernels). Odd rows take the TMA kernel
// when the planes' tensor map can be built (base and row stride 16-byte
// aligned, box of at most 256 words), else the cp.async kernel.
int launch_decode_recompose_nb32(const void* base, uint64_t stride, int planes, uint64_t nblocks, const void* maxkey,
                                 const uint8_t* dnum, const float* coarse, const Box& F, const Box& C, float* out,
                                 uint64_t s0, uint64_t s1, int* status, cudaStream_t st, bool pdl) {
    if (!decode_recompose_nb32_ok(F)) return PRODM_EUNSUPPORTED;
    const size_t smem = fused_smem(F);
    const bool odd = (F.n[2] & 1u) != 0;
    if (odd && status && (uintptr_t)base % 16 == 0 && stride % 4 == 0) {
        const uint32_t bw = (fused_max_blocks(F) + 3 + 3) & ~3u;   // block range + up to 3 words of alignment
        const int nd = ws_decode_warps();
        const uint32_t bwn = (ws_tile_blocks(F, nd) + 3 + 3) & ~3u;
        // rows of 257 values and up take the warp-specialised form with
        // 16 - nd rows per unit where its tile rows fit 192 words (two CTAs
        // per SM; level 6 at 513^3: 46.4 us against 48.9 us for the 8-warp
        // kernel); longer rows keep 8-row units
        if (nd != 8 && ((fused_ws() == 2 && F.n[2] >= 257) || fused_ws() == 1) && bwn <= 192) {
            const uint32_t rs = bwn <= 96 ? 96 : (bwn <= 160 ? 160 : 192);
            alignas(64) CUtensorMap map;
            const int tall =
                tma_tall() && planes <= 32 && encode_plane_map(&map, base, nblocks, planes, stride, rs, 32) == PRODM_OK;
            if (tall || encode_plane_map(&map, base, nblocks, planes, stride, bwn, 1) == PRODM_OK) {
#define PRODM_WS_CASE(R, N)                                                                                   \
    if (rs == R && nd == N)                                                                                   \
        return launch_fused_ws<R, N>(map, bwn, maxkey, dnum, coarse, F, C, out, s0, s1, status, st, pdl, tall);
                PRODM_WS_CASE(96, 5) PRODM_WS_CASE(160, 5) PRODM_WS_CASE(192, 5)
                PRODM_WS_CASE(96, 6) PRODM_WS_CASE(160, 6) PRODM_WS_CASE(192, 6)
#undef PRODM_WS_CASE
            }
        }
        if (bw <= 256) {
            const uint32_t rs = fused_tma_stride(bw);
            // tall: one box of rs words x 32 plane rows per unit (planes above
            // the retrieved ones at negative coordinates, zero filled); else one
            // box of bw words per retrieved plane
            alignas(64) CUtensorMap map;
            const int tall =
                tma_tall() && planes <= 32 && encode_plane_map(&map, base, nblocks, planes, stride, rs, 32) == PRODM_OK;
            if (tall || encode_plane_map(&map, base, nblocks, planes, stride, bw, 1) == PRODM_OK) {
                if (rs == 96)
                    return launch_fused_tma<96>(map, bw, maxkey, dnum, coarse, F, C, out, s0, s1, status, st, pdl, tall);
                if (rs == 160)
                    return launch_fused_tma<160>(map, bw, maxkey, dnum, coarse, F, C, out, s0, s1, status, st, pdl, tall);
                return launch_fused_tma<256>(map, bw, maxkey, dnum, coarse, F, C, out, s0, s1, status, st, pdl, tall);
            }
        }
    }
    const void* kern = odd ? (const void*)k_decode_recompose_nb32_odd : (const void*)k_decode_recompose_nb32;
    if (smem > 48 * 1024) {   // per device; cheap to repeat
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
        if (e != cudaSuccess) return cuda_status(e, "cudaFuncSetAttribute");
    }
    const uint64_t rows = (uint64_t)F.n[0] * F.n[1];
    const uint64_t need = (rows + 7) / 8;
    if (odd) {
        const unsigned grid = persistent_grid_for(kern, 256, smem, need, need);
        k_decode_recompose_nb32_odd<<<grid, 256, smem, st>>>((const uint32_t*)base, stride, (const uint32_t*)maxkey,
                                                             dnum, coarse, F, C, out, s0, s1, fused_max_blocks(F));
        PRODM_CHECK_LAUNCH("k_decode_recompose_nb32_odd");
        return PRODM_OK;
    }
    const unsigned grid = persistent_grid_for((const void*)k_decode_recompose_nb32, 256, smem, need, need);
    k_decode_recompose_nb32<<<grid, 256, smem, st>>>((const uint32_t*)base, stride, (const uint32_t*)maxkey, dnum,
                                                     coarse, F, C, out, s0, s1, fused_max_blocks(F));
    PRODM_CHECK_LAUNCH("k_decode_recompose_nb32");
    return PRODM_OK;
}

uint32_t fused_unit_blocks(const Box& F) { return fused_max_blocks(F); }

uint32_t fused_unit_rows(const Box& F, uint32_t values) {
    const uint32_t m = values / 8 / (F.n[2] ? F.n[2] : 1);
    return 8 * (m < 1 ? 1 : (m > kMaxUnitRows / 8 ? kMaxUnitRows / 8 : m));
}
uint32_t fused_unit_blocks_rows(const Box& F, uint32_t nr) { return (uint32_t)(((uint64_t)nr * F.n[2] + 31) / 32 + 2); }

uint32_t fused_tma_box(const Box& F, uint32_t nr) {
    if (!(F.n[2] & 1u)) return 0;
    const uint32_t bw = (fused_unit_blocks_rows(F, nr) + 3 + 3) & ~3u;   // block range + up to 3 words of alignment
    return bw <= 160 ? bw : 0;
}

int encode_plane_map(void* map, const void* base, uint64_t nblocks, int planes, uint64_t stride, uint32_t bw,
                     uint32_t box_planes) {
    PFN_cuTensorMapEncodeTiled_v12000 enc = tensor_map_encoder();
    if (!enc || !bw || (uintptr_t)base % 16 != 0 || stride % 4 != 0) return PRODM_EUNSUPPORTED;
    const cuuint64_t dims[2] = {nblocks, (cuuint64_t)planes};
    const cuuint64_t strides[1] = {stride * 4};
    const cuuint32_t box[2] = {bw, box_planes};
    const cuuint32_t estr[2] = {1, 1};
    if (enc((CUtensorMap*)map, CU_TENSOR_MAP_DATA_TYPE_UINT32, 2, const_cast<void*>(base), dims, strides, box, estr,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
        return PRODM_EUNSUPPORTED;
    return PRODM_OK;
}

template <int RS>
static int launch_tma_multi(const FusedSeg* segs, int nseg, uint64_t total_units, uint32_t tld, unsigned ctas_per_sm,
                            int* status, cudaStream_t st) {
    const size_t smem = (size_t)32 * RS * 4 + (size_t)tld * CB_LD * 4;
    const void* kern = (const void*)k_decode_recompose_nb32_tma_multi<RS>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return cuda_status(e, "cudaFuncSetAttribute");
    uint64_t cap = persistent_grid_for(kern, 256, smem, total_units, total_units);
    if (ctas_per_sm) cap = std::min<uint64_t>(cap, (uint64_t)device_sms() * ctas_per_sm);
    const unsigned grid = (unsigned)std::max<uint64_t>(cap, 1);
    k_decode_recompose_nb32_tma_multi<RS><<<grid, 256, smem, st>>>(segs, nseg, total_units, status, g_tma_wait_cycles,
                                                                  (uint32_t)g_tma_tx_extra);
    PRODM_CHECK_LAUNCH("k_decode_recompose_nb32_tma_multi");
    return PRODM_OK;
}

int launch_decode_recompose_nb32_tma_multi(const FusedSeg* segs, int nseg, uint64_t total_units, uint32_t tld,
                                           uint32_t max_bw, unsigned ctas_per_sm, int* status, cudaStream_t st) {
    if (!total_units) return PRODM_OK;
    if (max_bw <= 96) return launch_tma_multi<96>(segs, nseg, total_units, tld, ctas_per_sm, status, st);
    if (max_bw <= 160) return launch_tma_multi<160>(segs, nseg, total_units, tld, ctas_per_sm, status, st);
    return fail(PRODM_EUNSUPPORTED, "batched fused level: TMA box above 160 words");
}
uint32_t fused_ws_unit_rows() { return ws_unit_rows(5); }

int launch_decode_recompose_nb32_ws_multi(const FusedSeg* segs, int nseg, uint64_t total_units, uint32_t tld,
                                          int* status, cudaStream_t st) {
    if (!total_units) return PRODM_OK;
    constexpr int RS = kWsMultiStride;
    const size_t smem = (size_t)2 * 32 * RS * 4 + (size_t)2 * tld * CB_LD * 4;
    const void* kern = (const void*)k_decode_recompose_nb32_ws_multi<RS, 5>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return cuda_status(e, "cudaFuncSetAttribute");
    const unsigned grid = persistent_grid_for(kern, 512, smem, total_units, total_units);
    k_decode_recompose_nb32_ws_multi<RS, 5><<<grid, 512, smem, st>>>(segs, nseg, total_units, tld, status,
                                                                    g_tma_wait_cycles, (uint32_t)g_tma_tx_extra);
    PRODM_CHECK_LAUNCH("k_decode_recompose_nb32_ws_multi");
    return PRODM_OK;
}
size_t fused_multi_smem(uint32_t tld) { return (size_t)tld * TB_LD * 4 + (size_t)tld * CB_LD * 4; }

// ctas_per_sm == 0: as many as fit
int launch_decode_recompose_nb32_multi(const FusedSeg* segs, int nseg, uint64_t total_units, uint32_t tld,
                                       unsigned ctas_per_sm, cudaStream_t st) {
    if (!total_units) return PRODM_OK;
    const size_t smem = fused_multi_smem(tld);
    if (smem > 200 * 1024) return fail(PRODM_EUNSUPPORTED, "batched fused level: rows too long");
    const void* kern = (const void*)k_decode_recompose_nb32_multi;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return cuda_status(e, "cudaFuncSetAttribute");
    uint64_t cap = persistent_grid_for(kern, 256, smem, total_units, total_units);
    if (ctas_per_sm) cap = std::min<uint64_t>(cap, (uint64_t)device_sms() * ctas_per_sm);
    const unsigned grid = (unsigned)std::max<uint64_t>(cap, 1);
    k_decode_recompose_nb32_multi<<<grid, 256, smem, st>>>(segs, nseg, total_units, tld);
    PRODM_CHECK_LAUNCH("k_decode_recompose_nb32_multi");
    return PRODM_OK;
}

}  // namespace prodm
