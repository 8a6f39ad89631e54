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
#include "common.cuh"
#include "kernels.cuh"
#include "nbcodec.cuh"

namespace prodm {

namespace {

constexpr unsigned FULL = 0xffffffffu;

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
constexpr int CB_LD = 33;   // value-major coefficient rows: conflict-free both ways

__device__ __forceinline__ float cb_at(const float* cb, uint32_t r) { return cb[r + (r >> 5)]; }

// one fine row of odd length n = 2 c2n - 1; M01 = odd-dim mask over dims
// 0/1 (0: both coarse -> only odd nodes carry coefficients, ranks c;
// otherwise even node 2c has rank c and odd node 2c+1 rank c2n + c). The row
// is c2n - 1 column pairs (nodes 2c, 2c+1) and a last node 2(c2n - 1). Lane l
// handles the pairs 32k + l; the corner values of D column groups are in
// flight at once (a ring of D groups in registers, refilled as each group is
// used), so a row waits for the L2 latency about once instead of once per
// group. Groups in which every lane has a pair run without bounds checks, on
// pointers advanced once per D groups; the last node is written by lane 0.
template <int M01>
__device__ __forceinline__ void recompose_row_odd(const float* __restrict__ cb0, uint64_t cs0, uint64_t cs1,
                                                  uint32_t c2n, const float* __restrict__ cb, uint32_t rb0,
                                                  float* __restrict__ orow, int lane) {
    constexpr int NQ = M01 == 0 ? 1 : (M01 == 3 ? 4 : 2);
    constexpr int D = M01 == 3 ? 3 : 4;
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
    const float* pe = cb + re + (re >> 5);
    const float* po = cb + ro + (ro >> 5);
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
            pair(q, qn, pe + 33 * d, po + 33 * d, o + 64 * d);
            const bool more = (int)(32 * (k0 + d + D)) < lim;   // refill: group k + D
#pragma unroll
            for (int i = 0; i < NQ; i++) ring[d][i] = more ? __ldg(pc[i] + 32 * (d + D)) : 0.f;
        }
#pragma unroll
        for (int i = 0; i < NQ; i++) pc[i] += 32 * D;
        pe += 33 * D;
        po += 33 * D;
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
        if ((int)(32 * k) < plim) pair(q, qn, pe + 33 * d, po + 33 * d, o + 64 * d);
        const bool more = (int)(32 * (k + D)) < lim;
#pragma unroll
        for (int i = 0; i < NQ; i++) ring[d][i] = more ? __ldg(pc[i] + 32 * (d + D)) : 0.f;
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
        uint32_t R[32];
        const uint4* src = reinterpret_cast<const uint4*>(tile + t * TB_LD);
#pragma unroll
        for (int q = 0; q < 8; q++) {
            const uint4 w = src[q];
            R[31 - 4 * q] = w.x;
            R[30 - 4 * q] = w.y;
            R[29 - 4 * q] = w.z;
            R[28 - 4 * q] = w.w;
        }
        uint32_t a[16];
        transpose32_half(R, half, a);
#pragma unroll
        for (int v = 0; v < 16; v++) {
            const int32_t iv = nb_to_bin(a[v]);
            if constexpr (FAST) dst[v] = (float)iv * dscale;
            else dst[v] = neg ? -ldexpf((float)iv, exp - num) : ldexpf((float)iv, exp - num);
        }
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
    const uint32_t n2 = F.n[2], c2n = C.n[2];
    const uint64_t cs0 = (uint64_t)C.n[1] * C.n[2], cs1 = C.n[2];
    auto row_rank = [&](uint32_t rho, uint32_t& r0, uint32_t& r1, bool& cc, uint64_t& rbase, uint32_t& len) {
        r0 = rho / F.n[1];
        r1 = rho - r0 * F.n[1];
        cc = r0 < C.n[0] && r1 < C.n[1];
        rbase = level_rank(r0, r1, cc ? c2n : 0u, F, C);
        len = cc ? n2 - c2n : n2;
    };
    // block range [fb, fb + nbk) of the coefficients of rows [rho0, rho0 + 8)
    auto block_range = [&](uint32_t rho0, uint64_t& fb, uint32_t& nbk) {
        const uint32_t rho_last = min(rho0 + 7, rows - 1);
        uint32_t a0, a1, z0, z1, alen, zlen;
        bool acc_, zcc;
        uint64_t abase, zbase;
        row_rank(rho0, a0, a1, acc_, abase, alen);
        row_rank(rho_last, z0, z1, zcc, zbase, zlen);
        fb = abase >> 5;
        nbk = (uint32_t)(((zbase + zlen - 1) >> 5) - fb + 1);
    };
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
        if (rho < rows) {
            uint32_t r0, r1, len;
            bool cc;
            uint64_t rbase;
            row_rank(rho, r0, r1, cc, rbase, len);
            const uint32_t x0 = natural_of(r0, F.n[0], C.n[0]), x1 = natural_of(r1, F.n[1], C.n[1]);
            const int m01 = (is_coarse(x0, F.n[0]) ? 0 : 1) | (is_coarse(x1, F.n[1]) ? 0 : 2);
            const uint32_t c0 = (m01 & 1) ? (x0 >> 1) : r0;
            const uint32_t c1 = (m01 & 2) ? (x1 >> 1) : r1;
            const float* cb0 = coarse + c0 * cs0 + c1 * cs1;
            float* orow = out + x0 * s0 + x1 * s1;
            const uint32_t rb0 = (uint32_t)(rbase - fb * 32);
            switch (m01) {
                case 0: recompose_row_odd<0>(cb0, cs0, cs1, c2n, cb, rb0, orow, lane); break;
                case 1: recompose_row_odd<1>(cb0, cs0, cs1, c2n, cb, rb0, orow, lane); break;
                case 2: recompose_row_odd<2>(cb0, cs0, cs1, c2n, cb, rb0, orow, lane); break;
                default: recompose_row_odd<3>(cb0, cs0, cs1, c2n, cb, rb0, orow, lane); break;
            }
        }
    }
    cp_async_wait_all();
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

// Returns PRODM_EUNSUPPORTED when the shape does not suit the row mapping
// (the caller then runs the unfused kernels).
int launch_decode_recompose_nb32(const void* base, uint64_t stride, const void* maxkey, const uint8_t* dnum,
                                 const float* coarse, const Box& F, const Box& C, float* out, uint64_t s0, uint64_t s1,
                                 cudaStream_t st) {
    if (!decode_recompose_nb32_ok(F)) return PRODM_EUNSUPPORTED;
    const size_t smem = fused_smem(F);
    const bool odd = (F.n[2] & 1u) != 0;
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

}  // namespace prodm
