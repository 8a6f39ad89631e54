// Bitplane encoders / decoders and error collectors (sm_103a).
//
// Stream layout on the device ("aligned layout"): the words of plane p of a
// level start at plane[p] (word aligned). NegaBinary planes all hold
// ceil(n / block) words; grouped planes hold between 0 and 2 * nblocks words.
// The grouped encoder's per-block recording bitplanes (the u8 header of
// stream 0, GroupedBPEncoder.hpp:66-71) are kept in a separate rb array.
// pack.cu turns this into the reference level-file byte layout.
//
// Warp mapping: one warp per block of 32 (fp32, u32 words) or 64 (fp64, u64
// words: each lane holds elements lane and lane + 32) values; __ballot_sync
// transposes one bitplane of the block into one stream word; lane p then
// owns the word of plane p (and p + 32 for fp64).
#include <algorithm>
#include <mutex>
#include <type_traits>
#include <utility>
#include <vector>

#include "common.cuh"
#include "errtab.cuh"
#include "kernels.cuh"
#include "nbcodec.cuh"

namespace prodm {

namespace {

constexpr unsigned FULL = 0xffffffffu;

template <class T>
__device__ __forceinline__ int level_exp(const typename KeyOf<T>::type* maxkey, int exp_arg) {
    return maxkey ? frexp_exp(key_to_val(*maxkey, T())) : exp_arg;
}

// quantisation shared by the encoders
__device__ __forceinline__ int32_t trunc_fps(float v) { return (int32_t)v; }
__device__ __forceinline__ int64_t trunc_fps(double v) { return (int64_t)v; }

// ---------------------------------------------------------------------------
// per-thread error accumulators -> per-CTA partial tables (B+1 doubles each):
// a fixed butterfly per warp, then the warps' totals in warp order, so a
// table does not depend on scheduling
// ---------------------------------------------------------------------------
template <int NACC, class A>
__device__ void flush_errors(A (&acc)[NACC], int B, double* partial) {
    __shared__ double red[8][NACC];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int k = 0; k < NACC; k++) {
        double v = (double)acc[k];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(FULL, v, o);
        if (lane == 0) red[warp][k] = v;
    }
    __syncthreads();
    for (int k = threadIdx.x; k <= B && k < NACC; k += blockDim.x) {
        double v = 0;
        for (int w = 0; w < nw; w++) v += red[w][k];
        partial[(size_t)blockIdx.x * (B + 1) + k] = v;
    }
}

// NegaBinaryBPEncoder::collect_level_errors (NegaBinaryBPEncoder.hpp:231-239)
// in shifted units: acc[B] += m^2, acc[B-k] += (nb2bin(nb & (2^k-1)) + m)^2,
// acc[0] += shifted^2.
template <int NACC>
__device__ __forceinline__ void nb_errors(double (&acc)[NACC], uint64_t nb, double shifted, double m, int B) {
    acc[B < NACC ? B : NACC - 1] += m * m;
#pragma unroll
    for (int k = 1; k < NACC - 1; k++) {
        if (k < B) {
            double d = (double)nb_to_bin((uint64_t)(nb & ((1ull << k) - 1ull))) + m;
            acc[B - k] += d * d;
        }
    }
    acc[0] += shifted * shifted;
}
// GroupedBPEncoder::collect_level_errors (GroupedBPEncoder.hpp:324-335), a = |shifted|
template <int NACC>
__device__ __forceinline__ void gr_errors(double (&acc)[NACC], double a, int B) {
    uint64_t fp = (uint64_t)a;
    double m = a - (double)fp;
    acc[B < NACC ? B : NACC - 1] += m * m;
#pragma unroll
    for (int k = 1; k < NACC - 1; k++) {
        if (k < B) {
            double d = (double)(fp & ((1ull << k) - 1ull)) + m;
            acc[B - k] += d * d;
        }
    }
    acc[0] += a * a;
}

// per-lane accumulators of the fp64 tables and of the squared-error collector:
// double whatever the data type (the reference sums in double)
template <class T> struct Acc { using type = double; static constexpr int N = 33; };
template <> struct Acc<double> { using type = double; static constexpr int N = 65; };

// fp32 negabinary encoder without tables: grid-stride over NB_CHUNK-block chunks
__global__ void __launch_bounds__(256) k_nb_encode32(const float* __restrict__ x, uint64_t n,
                                                    const uint32_t* __restrict__ maxkey, int exp_arg, int B,
                                                    uint32_t* __restrict__ out, uint64_t stride) {
    __shared__ uint32_t tile[32 * NB_TILE_LD];
    const int exp = (maxkey ? frexp_exp(__uint_as_float(*maxkey)) : exp_arg) + 2;   // NegaBinaryBPEncoder.hpp:21
    const uint64_t nblocks = (n + 31) / 32;
    const uint64_t nchunks = (nblocks + NB_CHUNK - 1) / NB_CHUNK;
    const int se = B - exp;
    const bool fast = pow2_normal(se);
    const float scale = fast ? pow2f(se) : 1.f;
    for (uint64_t c = blockIdx.x; c < nchunks; c += gridDim.x)
        nb_encode32_chunk(x, n, nblocks, B, se, fast, scale, out, stride, c, tile);
}

// Every level of one fp32 field in one launch, without tables: segments are
// the levels in chunk order.
__global__ void __launch_bounds__(256, 3) k_nb_encode32_levels(const ChunkSeg* __restrict__ segs, int nseg,
                                                               uint64_t total, int B) {
    __shared__ uint32_t tile[32 * NB_TILE_LD];
    int cur = -1, se = 0;
    bool fast = true;
    float scale = 1.f;
    for (uint64_t c = blockIdx.x; c < total; c += gridDim.x) {
        const int s = find_seg(segs, nseg, c, &ChunkSeg::chunk_begin);
        const ChunkSeg& q = segs[s];
        if (s != cur) {
            cur = s;
            se = B - (frexp_exp(__uint_as_float(*q.key)) + 2);     // NegaBinaryBPEncoder.hpp:21
            fast = pow2_normal(se);
            scale = fast ? pow2f(se) : 1.f;
        }
        if (B == 32)
            nb_encode32_chunk<true>(q.x, q.n, q.nblocks, B, se, fast, scale, q.words, q.stride, c - q.chunk_begin, tile);
        else
            nb_encode32_chunk(q.x, q.n, q.nblocks, B, se, fast, scale, q.words, q.stride, c - q.chunk_begin, tile);
    }
}

// ---------------------------------------------------------------------------
// fp32 negabinary encoder with exact squared-error tables (errtab.cuh):
// NegaBinaryBPEncoder.hpp:65-125. Each lane takes four values per step (one
// from each of four consecutive blocks): their scaled values, negabinary
// digits and t = nb ^ 0xAAAAAAAA; the byte products of t go to the lane's
// exact sums, values below 2^23 to the warp's queue, and the four digit words
// are transposed into the plane tile (whose popcounts give the bit counts).
// ---------------------------------------------------------------------------
// plane tile of the table encoder: rows of ERR_LD words (16-byte aligned), so
// each lane stores its four transposed words of a step as one 16-byte store
// (conflict-free: rows differ by 65 16-byte units) and the chunk's plane runs
// leave with 16-byte copies
static_assert(errtab::kSlotsPad == kErrRecWords && errtab::WORDS + 16 <= errtab::kSlotsPad,
              "record width of the table encoders");
constexpr int ERR_LD = 260;
constexpr int kErrTileBytes = 32 * ERR_LD * 4;
constexpr size_t kErrSmemNB = (size_t)kErrTileBytes + 8 * sizeof(errtab::WarpQ) +
                              errtab::kSlotsPad * sizeof(unsigned long long);
// chunks a CTA encodes between two flushes of its 32-bit lane sums (each
// chunk adds at most 8 * 260100 to a lane sum)
constexpr int kErrFlushChunks = 2048;

// the 8 four-value steps of one warp over its 32 blocks; FULLW: every value
// of the blocks is inside the level (no bounds checks)
template <bool FULLB, bool FULLW>
__device__ __forceinline__ void nb_err_steps(const float* __restrict__ xw, int64_t rem, int B, int se, bool fast,
                                             float scale, uint32_t* trow, errtab::Lane& acc, errtab::WarpQ& wq,
                                             uint32_t& head, int& qn) {
    const int lane = threadIdx.x & 31;
    float vn[4];
    auto load4 = [&](int j0) {
#pragma unroll
        for (int g = 0; g < 4; g++) {
            const int o = (j0 + g) * 32;
            vn[g] = (FULLW || o < rem) ? __ldcs(xw + o) : 0.f;
        }
    };
    load4(0);
#pragma unroll 1
    for (int j0 = 0; j0 < 32; j0 += 4) {
        float sh[4];
        if (fast) {                                                 // NegaBinaryBPEncoder.hpp:42
#pragma unroll
            for (int g = 0; g < 4; g++) sh[g] = vn[g] * scale;
        } else {
#pragma unroll
            for (int g = 0; g < 4; g++) sh[g] = ldexpf(vn[g], se);
        }
        if (j0 + 4 < 32) load4(j0 + 4);                            // next step's values in flight
        uint32_t t[4], nb[4];
        bool small[4];
#pragma unroll
        for (int g = 0; g < 4; g++) {
            const bool ok = FULLW || (j0 + g) * 32 < rem;
            const uint32_t tq = (uint32_t)(int32_t)sh[g] + 0xaaaaaaaau;   // :43-44; nb = t ^ 0xAAAAAAAA
            nb[g] = tq ^ 0xaaaaaaaau;
            t[g] = ok ? tq : 0u;                                          // padding adds nothing
            const bool big = fabsf(sh[g]) >= 8388608.f;
            acc.add_big_square(sh[g], big);                               // padding is 0: never big
            small[g] = ok && !big;
        }
        errtab::enqueue4(wq, head, qn, small, sh, lane);
        errtab::drain_full<true>(wq, head, qn, lane);
        acc.add4(t[0], t[1], t[2], t[3]);
        uint32_t w[4];
#pragma unroll
        for (int g = 0; g < 4; g++) {
            w[g] = transpose32(nb[g], lane);
            acc.pc += __popc(w[g]);
        }
        if (FULLB || lane < B) *reinterpret_cast<uint4*>(trow + j0) = make_uint4(w[0], w[1], w[2], w[3]);
    }
}

template <bool FULLB>
__device__ __forceinline__ void nb_encode32_chunk_err(const float* __restrict__ x, uint64_t n, uint64_t nblocks, int B,
                                                      int se, bool fast, float scale, uint32_t* __restrict__ out,
                                                      uint64_t stride, uint64_t c, uint32_t* tile, errtab::Lane& acc,
                                                      errtab::WarpQ& wq, uint32_t& head, int& qn) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int plane = B - 1 - lane;      // lane k owns bit k = plane B-1-k
    const uint64_t cb0 = c * NB_CHUNK;
    const uint64_t v0 = (cb0 + (uint64_t)warp * 32) * 32;     // first value of the warp's 32 blocks
    const float* xw = x + v0 + lane;
    const int64_t rem = (int64_t)n - (int64_t)v0 - lane;      // this lane's values left in the level
    uint32_t* trow = tile + plane * ERR_LD + warp * 32;
    if ((int64_t)n - (int64_t)v0 >= 1024)                     // warp-uniform: all 32 blocks inside
        nb_err_steps<FULLB, true>(xw, rem, B, se, fast, scale, trow, acc, wq, head, qn);
    else
        nb_err_steps<FULLB, false>(xw, rem, B, se, fast, scale, trow, acc, wq, head, qn);
    __syncwarp();
    // the warp writes out its own 32 columns of the tile (blocks warp*32 ..
    // warp*32 + 31 of the chunk), so warps never wait for one another
    const int nvalid = (int)((nblocks - cb0) < (uint64_t)NB_CHUNK ? (nblocks - cb0) : NB_CHUNK);
    const int wb = warp * 32;
    if ((stride & 3) == 0 && (reinterpret_cast<uintptr_t>(out) & 15) == 0) {
        // 16-byte runs, four planes per instruction (8 lanes per plane); words
        // past nvalid are zero (blocks past the level) and land in the plane
        // row's padding to a multiple of four words
        const int nq = (nvalid + 3) >> 2;
        const int q = lane & 7;
        const bool ok = wb / 4 + q < nq;
#pragma unroll
        for (int p0 = 0; p0 < 32; p0 += 4) {
            const int p = p0 + (lane >> 3);
            if (p0 < B) {
                const uint4 v = reinterpret_cast<const uint4*>(tile + p * ERR_LD + wb)[q];
                if (ok && p < B) reinterpret_cast<uint4*>(out + (uint64_t)p * stride + cb0 + wb)[q] = v;
            }
        }
    } else {
        const bool ok = wb + lane < nvalid;
        for (int p = 0; p < B; p++) {
            const uint32_t v = tile[p * ERR_LD + wb + lane];
            if (ok) out[(uint64_t)p * stride + cb0 + wb + lane] = v;
        }
    }
    // the warp's own barrier (id 1 + warp, 32 threads) before its columns
    // are written again; as a barrier it also keeps the compiler from
    // interleaving the next chunk's loads with this copy (which spills)
    asm volatile("bar.sync %0, 32;" ::"r"(warp + 1) : "memory");
}

// Every level (segment) of one fp32 field with tables in one launch. Records
// (errtab::kSlotsPad u64 each) sit at recs + (level * gridDim.x + CTA); a CTA
// zeroes the record of every level it enters or skips and adds its sums at
// each level change, so every record the final reduction reads is written.
__global__ void __launch_bounds__(256, 2) k_nb_encode32_err(const ChunkSeg* __restrict__ segs, ChunkSeg one,
                                                            int nseg, uint64_t total, int B, int exp_arg,
                                                            unsigned long long* __restrict__ recs) {
    extern __shared__ __align__(16) unsigned char smem[];
    uint32_t* tile = (uint32_t*)smem;
    errtab::WarpQ* wq = (errtab::WarpQ*)(smem + kErrTileBytes);
    unsigned long long* red = (unsigned long long*)(wq + 8);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    errtab::Lane acc;
    acc.zero();
    errtab::zero_q(wq[warp], lane);
    uint32_t head = 0;
    int qn = 0;
    auto rec_of = [&](int s) { return recs + ((size_t)s * gridDim.x + blockIdx.x) * errtab::kSlotsPad; };
    auto zero_recs = [&](int s0, int s1) {   // levels [s0, s1)
        for (int s = s0; s < s1; s++)
            for (int k = threadIdx.x; k < errtab::kSlotsPad; k += blockDim.x) rec_of(s)[k] = 0;
        __syncthreads();
    };
    auto flush = [&](int s) {
        if (qn) {   // the queue's last partial batch
            __syncwarp();
            errtab::run_batch<true>(wq[warp], head, qn, lane);
            head += qn;
            qn = 0;
        }
        errtab::flush(acc, wq, red, rec_of(s));
    };
    int cur = -1, se = 0, since = 0;
    bool fast = true;
    float scale = 1.f;
    const float* qx = one.x;
    uint32_t* qw = one.words;
    uint64_t qnv = one.n, qnb = one.nblocks, qst = one.stride, qc0 = 0;
    // one flush site: at a level change, every kErrFlushChunks chunks, and at the end
    for (uint64_t c = blockIdx.x;; c += gridDim.x) {
        const bool done = c >= total;
        const int s = done ? nseg : (segs ? find_seg(segs, nseg, c, &ChunkSeg::chunk_begin) : 0);
        if (cur >= 0 && (s != cur || since == kErrFlushChunks)) {
            flush(cur);
            since = 0;
        }
        if (s != cur) {
            zero_recs(cur + 1, s < nseg ? s + 1 : nseg);
            if (done) break;
            cur = s;
            const uint32_t* key = one.key;
            if (segs) {
                qx = segs[s].x;
                qw = segs[s].words;
                qnv = segs[s].n;
                qnb = segs[s].nblocks;
                qst = segs[s].stride;
                qc0 = segs[s].chunk_begin;
                key = segs[s].key;
            }
            se = B - ((key ? frexp_exp(__uint_as_float(*key)) : exp_arg) + 2);   // NegaBinaryBPEncoder.hpp:21
            fast = pow2_normal(se);
            scale = fast ? pow2f(se) : 1.f;
        }
        since++;
        if (B == 32)
            nb_encode32_chunk_err<true>(qx, qnv, qnb, B, se, fast, scale, qw, qst, c - qc0, tile, acc, wq[warp], head,
                                        qn);
        else
            nb_encode32_chunk_err<false>(qx, qnv, qnb, B, se, fast, scale, qw, qst, c - qc0, tile, acc, wq[warp], head,
                                         qn);
    }
}

// Tables of every level from the CTA records: one CTA of 1024 threads per
// level. Thread (k, i), k < 5, sums record word i over records k, k + 5, ..
// (loads of all words in flight at once; low words of 128-bit sums also
// count their carries), then thread i combines the five partial sums in k
// order (so the doubles are summed in a fixed order) and thread i <= B
// computes entry i. keys (or exp_arg when keys is null) give the level
// exponent, exp_add the encoder's offset (2 for negabinary).
constexpr int kFinalParts = 5;
static_assert(kFinalParts * errtab::kSlotsPad <= 1024, "one thread per (part, record word)");

template <bool NB>
__global__ void __launch_bounds__(1024) k_errtab_final(const unsigned long long* __restrict__ recs, int nrec, int B,
                                                       const ChunkSeg* __restrict__ segs, ChunkSeg one, int exp_arg,
                                                       int exp_add, double* __restrict__ out) {
    __shared__ unsigned long long P[kFinalParts][errtab::kSlotsPad];    // partial sums (u64 words or double bits)
    __shared__ unsigned long long Cy[kFinalParts][errtab::kSlotsPad];   // carries out of the low words
    __shared__ unsigned long long R[errtab::kSlotsPad];
    const int l = blockIdx.x;
    const unsigned long long* rl = recs + (size_t)l * nrec * errtab::kSlotsPad;
    const int t = threadIdx.x;
    if (t < kFinalParts * errtab::kSlotsPad) {
        const int k = t / errtab::kSlotsPad, i = t - k * errtab::kSlotsPad;
        if (i < errtab::WORDS) {
            const unsigned long long* p = rl + i;
            if (errtab::slot_kind(i) == 3) {
                double v = 0;
#pragma unroll 8
                for (int r = k; r < nrec; r += kFinalParts) v += __longlong_as_double(p[(size_t)r * errtab::kSlotsPad]);
                P[k][i] = __double_as_longlong(v);
            } else {
                unsigned long long v = 0, c = 0;
#pragma unroll 8
                for (int r = k; r < nrec; r += kFinalParts) {
                    const unsigned long long o = v;
                    v += p[(size_t)r * errtab::kSlotsPad];
                    c += v < o ? 1 : 0;
                }
                P[k][i] = v;
                Cy[k][i] = c;
            }
        }
    }
    __syncthreads();
    if (t < errtab::WORDS) {
        const int kind = errtab::slot_kind(t);
        if (kind == 3) {
            double v = 0;
            for (int k = 0; k < kFinalParts; k++) v += __longlong_as_double(P[k][t]);
            R[t] = __double_as_longlong(v);
        } else if (kind != 2) {
            unsigned long long v = 0, c = 0;
            for (int k = 0; k < kFinalParts; k++) {
                const unsigned long long o = v;
                v += P[k][t];
                c += Cy[k][t] + (v < o ? 1 : 0);
            }
            R[t] = v;
            Cy[0][t] = c;   // carries into the high word (read by thread t + 1 after the barrier)
        }
    }
    __syncthreads();
    if (t < errtab::WORDS && errtab::slot_kind(t) == 2) {
        unsigned long long v = Cy[0][t - 1];
        for (int k = 0; k < kFinalParts; k++) v += P[k][t];
        R[t] = v;
    }
    __syncthreads();
    const uint32_t* key = segs ? segs[l].key : one.key;
    const uint64_t n = segs ? segs[l].n : one.n;
    const int e = (key ? frexp_exp(__uint_as_float(*key)) : exp_arg) + exp_add;
    for (int i = t; i <= B; i += blockDim.x) out[(size_t)l * (B + 1) + i] = errtab::table_entry<NB>(R, n, B, e, i);
}

// Every level of one fp32 field decoded in one launch (segments = levels in
// chunk order, kDecodeChunkBlocks 32-value blocks per chunk). Plane rows start
// on 16-byte boundaries, so a chunk's run of one plane (512 bytes) is one
// warp-wide 16-byte cp.async; the next chunk's planes are fetched into the
// second [plane][block] tile while the current chunk is decoded. Each
// 32-value block is decoded by two threads (one half transpose each), and a
// thread writes its 16 values as four 16-byte stores when the level's output
// is 16-byte aligned. NegaBinaryBPEncoder.hpp:132-192 with start plane 0 and
// num = dnum planes.
constexpr int DEC_LD = kDecodeChunkBlocks + 4;   // tile row (words): 16-byte aligned, conflict-free columns

__global__ void __launch_bounds__(256) k_nb_decode_levels(const ChunkSeg* __restrict__ segs, int nseg,
                                                         uint64_t total) {
    constexpr int CB = kDecodeChunkBlocks;
    __shared__ __align__(16) uint32_t tiles[2][32 * DEC_LD];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    pdl_wait();   // plane counts from the interpreter
    pdl_release();
    auto fetch = [&](uint64_t c, uint32_t* tile) {
        const ChunkSeg& q = segs[find_seg(segs, nseg, c, &ChunkSeg::chunk_begin)];
        const int num = q.dnum[0];
        const uint64_t b0 = (c - q.chunk_begin) * CB;
        const uint32_t nb = (uint32_t)min((uint64_t)CB, q.nblocks - b0);
        const uint32_t nq = (nb + 3) / 4;     // 16-byte pieces (inside the padded row)
        for (int p = warp; p < num; p += 8) {
            const uint32_t* src = q.words + (uint64_t)p * q.stride + b0;
            for (uint32_t j = lane; j < nq; j += 32) cp_async16(tile + p * DEC_LD + 4 * j, src + 4 * j);
        }
        cp_async_commit();
    };
    uint64_t c = blockIdx.x;
    if (c >= total) return;
    fetch(c, tiles[0]);
    for (int it = 0; c < total; it++, c += gridDim.x) {
        cp_async_wait_all();
        __syncthreads();
        if (c + gridDim.x < total) fetch(c + gridDim.x, tiles[(it + 1) & 1]);
        const uint32_t* tile = tiles[it & 1];
        const ChunkSeg& q = segs[find_seg(segs, nseg, c, &ChunkSeg::chunk_begin)];
        const int num = q.dnum[0];
        const uint64_t b0 = (c - q.chunk_begin) * CB;
        const uint32_t nb = (uint32_t)min((uint64_t)CB, q.nblocks - b0);
        const uint32_t t = threadIdx.x >> 1;
        const int half = threadIdx.x & 1;
        if (t < nb) {
            float vals[16];
            if (num == 0) {
#pragma unroll
                for (int v = 0; v < 16; v++) vals[v] = 0.f;
            } else {
                const int exp = frexp_exp(__uint_as_float(*q.key)) + 2;      // NegaBinaryBPEncoder.hpp:21
                const bool neg = num & 1;                                     // :153, :177
                const bool dfast = pow2_normal(exp - num);
                const float dscale = dfast ? (neg ? -pow2f(exp - num) : pow2f(exp - num)) : 1.f;
                // rows in reverse plane order: value v's digits come out most significant first
                uint32_t R[32];
#pragma unroll
                for (int p = 0; p < 32; p++) R[31 - p] = p < num ? tile[p * DEC_LD + t] : 0u;
                uint32_t a[16];
                transpose32_half(R, half, a);
#pragma unroll
                for (int v = 0; v < 16; v++) {
                    const int32_t iv = nb_to_bin(a[v] >> (32 - num));
                    vals[v] = dfast ? (float)iv * dscale
                                    : (neg ? -ldexpf((float)iv, exp - num) : ldexpf((float)iv, exp - num));
                }
            }
            const uint64_t e0 = (b0 + t) * 32 + 16 * (uint64_t)half;
            float* dst = q.y + e0;
            if (e0 + 16 <= q.n && ((reinterpret_cast<uintptr_t>(dst) & 15u) == 0)) {
                float4* d4 = reinterpret_cast<float4*>(dst);
#pragma unroll
                for (int k = 0; k < 4; k++) d4[k] = make_float4(vals[4 * k], vals[4 * k + 1], vals[4 * k + 2], vals[4 * k + 3]);
            } else {
#pragma unroll
                for (int v = 0; v < 16; v++)
                    if (e0 + v < q.n) dst[v] = vals[v];
            }
        }
    }
    cp_async_wait_all();
}

// fp32 negabinary decoder, planes [s, s+num) at base[i * stride]
__global__ void __launch_bounds__(256) k_nb_decode32(const uint32_t* __restrict__ base, uint64_t stride, uint64_t n,
                                                    const uint32_t* __restrict__ maxkey, int exp_arg, int s, int num,
                                                    const uint8_t* __restrict__ dnum, float* __restrict__ out) {
    __shared__ uint32_t tile[32 * NB_TILE_LD];
    if (dnum) num = dnum[0] - s;
    const int exp = (maxkey ? frexp_exp(__uint_as_float(*maxkey)) : exp_arg) + 2;
    const int e = s + num;
    const uint64_t nblocks = (n + 31) / 32;
    const uint64_t nchunks = (nblocks + NB_CHUNK - 1) / NB_CHUNK;
    const bool dfast = pow2_normal(exp - e);
    const float dscale = dfast ? pow2f(exp - e) : 1.f;
    for (uint64_t c = blockIdx.x; c < nchunks; c += gridDim.x)
        nb_decode32_chunk(base, stride, n, nblocks, num, e, exp, dfast, dscale, c, tile, out);
}

// ---------------------------------------------------------------------------
// NegaBinary encoder -- NegaBinaryBPEncoder.hpp:18-62 (+ :65-125 errors)
// ---------------------------------------------------------------------------
template <class T, bool ERR>
__global__ void __launch_bounds__(256) k_nb_encode(const T* __restrict__ x, uint64_t n,
                                                   const typename KeyOf<T>::type* __restrict__ maxkey, int exp_arg,
                                                   int B, typename Traits<T>::S* __restrict__ out, uint64_t stride,
                                                   double* __restrict__ partial) {
    using S = typename Traits<T>::S;
    using FPS = typename Traits<T>::FPS;
    using FP = typename Traits<T>::FP;
    using A = typename Acc<T>::type;
    constexpr int BS = Traits<T>::kBlock;
    const int exp = level_exp<T>(maxkey, exp_arg) + 2;   // :21
    const int lane = threadIdx.x & 31;
    const uint64_t nblocks = (n + BS - 1) / BS;
    const uint64_t warps = (uint64_t)gridDim.x * (blockDim.x >> 5);
    A acc[Acc<T>::N];
    if (ERR) {
#pragma unroll
        for (int k = 0; k < Acc<T>::N; k++) acc[k] = 0;
    }
    for (uint64_t b = (uint64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); b < nblocks; b += warps) {
        FP nb[BS / 32];
#pragma unroll
        for (int h = 0; h < BS / 32; h++) {
            uint64_t i = b * BS + h * 32 + lane;
            nb[h] = 0;
            if (i < n) {
                T shifted = ldexp_t(x[i], B - exp);          // :42
                FPS q = trunc_fps(shifted);
                nb[h] = nb_from_bin(q);
                if (ERR) nb_errors(acc, nb[h], (A)shifted, (A)(shifted - (T)q), B);
            }
        }
        S mine0 = 0, mine1 = 0;
        for (int p = 0; p < B; p++) {                        // encode_block :240-250
            const int k = B - 1 - p;
            S w = (S)__ballot_sync(FULL, (nb[0] >> k) & 1u);
            if (BS == 64) w |= (S)__ballot_sync(FULL, (nb[BS / 32 - 1] >> k) & 1u) << (BS == 64 ? 32 : 0);
            if ((p & 31) == lane) {
                if (p < 32) mine0 = w; else mine1 = w;
            }
        }
        if (lane < B) out[(uint64_t)lane * stride + b] = mine0;
        if (lane + 32 < B) out[(uint64_t)(lane + 32) * stride + b] = mine1;
    }
    if (ERR) flush_errors(acc, B, partial);
}

// NegaBinaryBPEncoder::progressive_decode -- :132-192. planes [s, s+num)
// with plane (s+i) at base[i * stride]; a device count (dnum[0]) overrides num.
template <class T>
__global__ void __launch_bounds__(256) k_nb_decode(const typename Traits<T>::S* __restrict__ base, uint64_t stride,
                                                   uint64_t n, const typename KeyOf<T>::type* __restrict__ maxkey,
                                                   int exp_arg, int s, int num, const uint8_t* __restrict__ dnum,
                                                   T* __restrict__ out) {
    using S = typename Traits<T>::S;
    using FP = typename Traits<T>::FP;
    constexpr int BS = Traits<T>::kBlock;
    if (dnum) num = dnum[0] - s;
    const int exp = level_exp<T>(maxkey, exp_arg) + 2;
    const int e = s + num;
    const int lane = threadIdx.x & 31;
    const uint64_t nblocks = (n + BS - 1) / BS;
    const uint64_t warps = (uint64_t)gridDim.x * (blockDim.x >> 5);
    for (uint64_t b = (uint64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); b < nblocks; b += warps) {
        S w0 = 0, w1 = 0;
        if (lane < num) w0 = __ldg(base + (uint64_t)lane * stride + b);
        if (lane + 32 < num) w1 = __ldg(base + (uint64_t)(lane + 32) * stride + b);
        FP acc[BS / 32];
#pragma unroll
        for (int h = 0; h < BS / 32; h++) acc[h] = 0;
        for (int i = 0; i < num; i++) {                       // decode_block :251-260
            S w = __shfl_sync(FULL, i < 32 ? w0 : w1, i & 31);
            const int k = num - 1 - i;
#pragma unroll
            for (int h = 0; h < BS / 32; h++) acc[h] |= (FP)((w >> (h * 32 + lane)) & 1u) << k;
        }
#pragma unroll
        for (int h = 0; h < BS / 32; h++) {
            uint64_t i = b * BS + h * 32 + lane;
            if (i < n) {
                T v = num == 0 ? (T)0 : ldexp_t((T)nb_to_bin(acc[h]), -e + exp);
                out[i] = (num != 0 && (e & 1)) ? -v : v;       // :153, :177
            }
        }
    }
}

// ---------------------------------------------------------------------------
// Grouped encoder -- GroupedBPEncoder.hpp:18-73 (+ :76-145 errors)
// Chunk = 8 warps x 32 blocks per CTA.
// ---------------------------------------------------------------------------
constexpr int GR_WARPS = 8;
constexpr int GR_BPW = 32;                       // blocks per warp
constexpr int GR_CHUNK = GR_WARPS * GR_BPW;      // blocks per CTA

// |trunc(ldexp(v, B - exp))| and the sign (GroupedBPEncoder.hpp:41-42). For
// doubles whose scaled value is not needed (SH false: no error tables) the
// magnitude comes from the bits with integer operations (fixed_mag).
template <class T, bool SH = true>
__device__ __forceinline__ typename Traits<T>::FP gr_mag(T v, int B, int exp, bool& neg, T& shifted) {
    if constexpr (std::is_same<T, double>::value && !SH) {
        neg = below_zero(v);
        return fixed_mag(v, B - exp);
    } else {
        shifted = ldexp_t(v, B - exp);                  // :41
        int64_t fix = (int64_t)shifted;                 // :42
        neg = v < 0;
        return (typename Traits<T>::FP)(neg ? -fix : fix);
    }
}

// ldexp((T)acc, s), negated when neg (GroupedBPEncoder.hpp:359-368); for
// doubles with a normal result by integer operations (fixed_value)
template <class T>
__device__ __forceinline__ T gr_value(typename Traits<T>::FP acc, int s, bool neg) {
    if constexpr (std::is_same<T, double>::value) {
        if (fixed_value_normal(s)) {
            const long long b = __double_as_longlong(fixed_value(acc, s));
            return __longlong_as_double(neg ? b ^ (long long)0x8000000000000000ull : b);
        }
    }
    const T v = ldexp_t((T)acc, s);
    return neg ? -v : v;
}

// word counts contributed by a block with recording plane r to plane p
__device__ __forceinline__ uint32_t gr_words(int r, int p) { return (r < p ? 1u : 0u) + (r == p ? 2u : 0u); }

template <class T, bool ERR>
__global__ void __launch_bounds__(256) k_gr_rb(const T* __restrict__ x, uint64_t n,
                                               const typename KeyOf<T>::type* __restrict__ maxkey, int exp_arg, int B,
                                               uint8_t* __restrict__ rbs, uint32_t* __restrict__ chunk_words,
                                               double* __restrict__ partial) {
    using FP = typename Traits<T>::FP;
    using A = typename Acc<T>::type;
    constexpr int BS = Traits<T>::kBlock;
    const int exp = level_exp<T>(maxkey, exp_arg);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint64_t nblocks = (n + BS - 1) / BS;
    __shared__ uint32_t cnt[GR_WARPS][64];
    uint32_t c0 = 0, c1 = 0;
    A acc[Acc<T>::N];
    if (ERR) {
#pragma unroll
        for (int k = 0; k < Acc<T>::N; k++) acc[k] = 0;
    }
    const uint64_t b0 = (uint64_t)blockIdx.x * GR_CHUNK + (uint64_t)warp * GR_BPW;
    for (int j = 0; j < GR_BPW; j++) {
        uint64_t b = b0 + j;
        if (b >= nblocks) break;
        FP orv = 0;
#pragma unroll
        for (int h = 0; h < BS / 32; h++) {
            uint64_t i = b * BS + h * 32 + lane;
            if (i < n) {
                bool neg;
                T sh;
                FP q = gr_mag<T, ERR>(x[i], B, exp, neg, sh);
                orv |= q;
                if (ERR) gr_errors(acc, (A)fabs(sh), B);
            }
        }
        int r;
        if (BS == 32) {
            uint32_t o = __reduce_or_sync(FULL, (uint32_t)orv);
            r = o ? B - 1 - (31 - __clz(o)) : B;
        } else {
            uint32_t lo = __reduce_or_sync(FULL, (uint32_t)orv);
            uint32_t hi = __reduce_or_sync(FULL, (uint32_t)((uint64_t)orv >> 32));
            uint64_t o = ((uint64_t)hi << 32) | lo;
            r = o ? B - 1 - (63 - __clzll((long long)o)) : B;
        }
        if (lane == 0) rbs[b] = (uint8_t)r;
        c0 += gr_words(r, lane);
        c1 += gr_words(r, lane + 32);
    }
    cnt[warp][lane] = c0;
    cnt[warp][lane + 32] = c1;
    __syncthreads();
    if (threadIdx.x < 64 && (int)threadIdx.x < B) {
        uint32_t s = 0;
        for (int w = 0; w < GR_WARPS; w++) s += cnt[w][threadIdx.x];
        chunk_words[(uint64_t)blockIdx.x * B + threadIdx.x] = s;
    }
    if (ERR) flush_errors(acc, B, partial);
}

// exclusive scan of chunk_words over chunks, per plane; stream byte sizes.
// One CTA per plane (the planes are independent).
__global__ void k_gr_scan(const uint32_t* __restrict__ chunk_words, uint64_t nchunks, int B, uint64_t nblocks,
                          int word_bytes, uint32_t* __restrict__ chunk_off, uint32_t* __restrict__ sizes) {
    __shared__ uint32_t wsum[32];
    __shared__ uint32_t carry;
    {
        const int p = blockIdx.x;
        if (p >= B) return;
        if (threadIdx.x == 0) carry = 0;
        __syncthreads();
        for (uint64_t base = 0; base < nchunks; base += blockDim.x) {
            uint64_t c = base + threadIdx.x;
            uint32_t v = c < nchunks ? chunk_words[c * B + p] : 0;
            uint32_t incl = v;
            const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                uint32_t t = __shfl_up_sync(FULL, incl, o);
                if (lane >= o) incl += t;
            }
            if (lane == 31) wsum[warp] = incl;
            __syncthreads();
            if (warp == 0) {
                uint32_t ws = lane < (int)(blockDim.x >> 5) ? wsum[lane] : 0;
                uint32_t wi = ws;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    uint32_t t = __shfl_up_sync(FULL, wi, o);
                    if (lane >= o) wi += t;
                }
                wsum[lane] = wi - ws;   // exclusive warp offsets
            }
            __syncthreads();
            uint32_t excl = carry + wsum[warp] + incl - v;
            if (c < nchunks) chunk_off[c * B + p] = excl;
            __syncthreads();
            if (threadIdx.x == blockDim.x - 1) carry = excl + v;
            __syncthreads();
        }
        if (threadIdx.x == 0) sizes[p] = carry * word_bytes + (p == 0 ? (uint32_t)(4 + nblocks) : 0u);
        __syncthreads();
    }
}

// per-warp starting offsets (word index in each plane) for the warp's 32 blocks
__device__ __forceinline__ void gr_warp_offsets(const uint8_t* __restrict__ rbs, uint64_t nblocks,
                                                const uint32_t* __restrict__ chunk_off, int B, uint32_t& off0,
                                                uint32_t& off1) {
    __shared__ uint32_t cnt[GR_WARPS][64];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint64_t b0 = (uint64_t)blockIdx.x * GR_CHUNK + (uint64_t)warp * GR_BPW;
    uint32_t c0 = 0, c1 = 0;
    for (int j = 0; j < GR_BPW; j++) {
        uint64_t b = b0 + j;
        if (b >= nblocks) break;
        int r = rbs[b];
        c0 += gr_words(r, lane);
        c1 += gr_words(r, lane + 32);
    }
    cnt[warp][lane] = c0;
    cnt[warp][lane + 32] = c1;
    __syncthreads();
    off0 = lane < B ? chunk_off[(uint64_t)blockIdx.x * B + lane] : 0;
    off1 = lane + 32 < B ? chunk_off[(uint64_t)blockIdx.x * B + lane + 32] : 0;
    for (int w = 0; w < warp; w++) {
        off0 += cnt[w][lane];
        off1 += cnt[w][lane + 32];
    }
}

template <class T>
__global__ void __launch_bounds__(256, 4) k_gr_write(const T* __restrict__ x, uint64_t n,
                                                  const typename KeyOf<T>::type* __restrict__ maxkey, int exp_arg,
                                                  int B, const uint8_t* __restrict__ rbs,
                                                  const uint32_t* __restrict__ chunk_off,
                                                  typename Traits<T>::S* __restrict__ out, uint64_t cap) {
    using S = typename Traits<T>::S;
    using FP = typename Traits<T>::FP;
    constexpr int BS = Traits<T>::kBlock;
    const int exp = level_exp<T>(maxkey, exp_arg);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint64_t nblocks = (n + BS - 1) / BS;
    uint32_t off0, off1;
    gr_warp_offsets(rbs, nblocks, chunk_off, B, off0, off1);
    const uint64_t b0 = (uint64_t)blockIdx.x * GR_CHUNK + (uint64_t)warp * GR_BPW;
    for (int j = 0; j < GR_BPW; j++) {
        uint64_t b = b0 + j;
        if (b >= nblocks) break;
        FP q[BS / 32];
        S sign = 0;
#pragma unroll
        for (int h = 0; h < BS / 32; h++) {
            uint64_t i = b * BS + h * 32 + lane;
            bool neg = false;
            q[h] = 0;
            if (i < n) {
                T sh;
                q[h] = gr_mag<T, false>(x[i], B, exp, neg, sh);
            }
            sign |= (S)__ballot_sync(FULL, neg) << (h * 32);
        }
        const int r = rbs[b];
        S mine0 = 0, mine1 = 0;
        if constexpr (BS == 64) {
            // encode_block :337-357 by four warp bit transposes: lane k gets the
            // words of magnitude bit k (low halves) and bit 32 + k (high halves)
            // of values 0..31 and 32..63; lane p then fetches plane p (bit
            // B-1-p) and plane p + 32 (bit B-33-p). Planes below r are not written.
            const uint32_t lo0 = transpose32((uint32_t)q[0], lane), hi0 = transpose32((uint32_t)(q[0] >> 32), lane);
            const uint32_t lo1 = transpose32((uint32_t)q[1], lane), hi1 = transpose32((uint32_t)(q[1] >> 32), lane);
            S w[2];
#pragma unroll
            for (int t = 0; t < 2; t++) {   // plane lane + 32 t (a valid plane for the shuffles' sake)
                const int p = lane + 32 * t < B ? lane + 32 * t : 0;
                const int k = B - 1 - p, src = k & 31;
                const uint32_t a0 = __shfl_sync(FULL, lo0, src), b0 = __shfl_sync(FULL, hi0, src);
                const uint32_t a1 = __shfl_sync(FULL, lo1, src), b1 = __shfl_sync(FULL, hi1, src);
                w[t] = k >= 32 ? ((S)b1 << 32 | b0) : ((S)a1 << 32 | a0);
            }
            mine0 = lane >= r ? w[0] : 0;
            mine1 = lane + 32 >= r ? w[1] : 0;
        } else {
            for (int p = r; p < B; p++) {                      // encode_block :337-357
                const int k = B - 1 - p;
                S w = (S)__ballot_sync(FULL, (q[0] >> k) & 1u);
                if ((p & 31) == lane) {
                    if (p < 32) mine0 = w; else mine1 = w;
                }
            }
        }
        if (lane < B && lane >= r) {
            S* dst = out + (uint64_t)lane * cap + off0;
            if (lane == r) { dst[0] = sign; dst[1] = mine0; }
            else dst[0] = mine0;
        }
        if (lane + 32 < B && lane + 32 >= r) {
            S* dst = out + (uint64_t)(lane + 32) * cap + off1;
            if (lane + 32 == r) { dst[0] = sign; dst[1] = mine1; }
            else dst[0] = mine1;
        }
        off0 += gr_words(r, lane);
        off1 += gr_words(r, lane + 32);
    }
}

// fp32 grouped writer: one transpose per block instead of B ballots. With
// ERR, the exact squared-error tables (errtab.cuh, GroupedBPEncoder.hpp:76-145
// with collect_level_errors :324-335) of the CTA's chunk go to its record
// recs + blockIdx.x: four blocks per step, t = trunc(|x|), bit counts from the
// transposed magnitude words.
constexpr size_t kErrSmemGR = 8 * sizeof(errtab::WarpQ) + errtab::kSlotsPad * sizeof(unsigned long long);

template <bool ERR>
__global__ void __launch_bounds__(256) k_gr_write32(const float* __restrict__ x, uint64_t n,
                                                   const uint32_t* __restrict__ maxkey, int exp_arg, int B,
                                                   const uint8_t* __restrict__ rbs,
                                                   const uint32_t* __restrict__ chunk_off, uint32_t* __restrict__ out,
                                                   uint64_t cap, unsigned long long* __restrict__ recs) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int exp = maxkey ? frexp_exp(__uint_as_float(*maxkey)) : exp_arg;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint64_t nblocks = (n + 31) / 32;
    uint32_t off0, off1;
    gr_warp_offsets(rbs, nblocks, chunk_off, B, off0, off1);
    const int plane = B - 1 - lane;                    // lane k owns bit k
    uint32_t off = __shfl_sync(FULL, off0, plane & 31);
    const bool fast = pow2_normal(B - exp);
    const float sc = fast ? pow2f(B - exp) : 1.f;
    const uint64_t b0 = (uint64_t)blockIdx.x * GR_CHUNK + (uint64_t)warp * GR_BPW;
    errtab::WarpQ* wq = (errtab::WarpQ*)smem;
    unsigned long long* red = (unsigned long long*)(wq + 8);
    errtab::Lane acc;
    uint32_t head = 0;
    int qn = 0;
    if (ERR) {
        acc.zero();
        errtab::zero_q(wq[warp], lane);
    }
    for (int j0 = 0; j0 < GR_BPW; j0 += 4) {
        float sh[4], mag[4];
        uint32_t q[4], sign[4];
        bool small[4];
#pragma unroll
        for (int g = 0; g < 4; g++) {
            const uint64_t i = (b0 + j0 + g) * 32 + lane;
            const bool ok = i < n;
            const float v = ok ? __ldcs(x + i) : 0.f;
            sh[g] = scale2(v, B - exp, fast, sc);
            const int64_t fix = (int64_t)sh[g];
            const bool neg = v < 0.f;
            q[g] = (uint32_t)(neg ? -fix : fix);
            sign[g] = __ballot_sync(FULL, neg);
            if (ERR) {
                mag[g] = fabsf(sh[g]);
                const bool big = mag[g] >= 8388608.f;
                acc.add_big_square(mag[g], big);                              // padding is 0: never big
                small[g] = ok && !big;
            }
        }
        if (ERR) {
            errtab::enqueue4(wq[warp], head, qn, small, mag, lane);
            errtab::drain_full<false>(wq[warp], head, qn, lane);
            acc.add4(q[0], q[1], q[2], q[3]);
        }
#pragma unroll
        for (int g = 0; g < 4; g++) {
            const uint64_t b = b0 + j0 + g;
            const uint32_t w = transpose32(q[g], lane);
            if (ERR) acc.pc += __popc(w);
            if (b < nblocks) {
                const int r = rbs[b];
                if (lane < B && plane >= r) {
                    uint32_t* dst = out + (uint64_t)plane * cap + off;
                    if (plane == r) { dst[0] = sign[g]; dst[1] = w; }
                    else dst[0] = w;
                }
                off += gr_words(r, plane);
            }
        }
    }
    if (ERR) {
        if (qn) {
            __syncwarp();
            errtab::run_batch<false>(wq[warp], head, qn, lane);
        }
        unsigned long long* rec = recs + (size_t)blockIdx.x * errtab::kSlotsPad;
        for (int k = threadIdx.x; k < errtab::kSlotsPad; k += blockDim.x) rec[k] = 0;
        __syncthreads();
        errtab::flush(acc, wq, red, rec);
    }
}

// fp32 grouped decoder, planes [s, e): lane p loads plane p's word of the block
__global__ void __launch_bounds__(256) k_gr_decode32(const uint32_t* const* __restrict__ planes, uint64_t n,
                                                    const uint32_t* __restrict__ maxkey, int exp_arg, int B, int s,
                                                    int e, const uint8_t* __restrict__ dnum,
                                                    const uint8_t* __restrict__ rbs,
                                                    const uint32_t* __restrict__ chunk_off,
                                                    uint32_t* __restrict__ signs, float* __restrict__ out) {
    if (dnum) e = dnum[0];
    const int exp = maxkey ? frexp_exp(__uint_as_float(*maxkey)) : exp_arg;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint64_t nblocks = (n + 31) / 32;
    uint32_t off0, off1;
    gr_warp_offsets(rbs, nblocks, chunk_off, B, off0, off1);
    const uint32_t* src = (lane < B && lane >= s && lane < e) ? planes[lane] : nullptr;
    const bool fast = pow2_normal(exp - e);
    const float sc = fast ? pow2f(exp - e) : 1.f;
    const uint64_t b0 = (uint64_t)blockIdx.x * GR_CHUNK + (uint64_t)warp * GR_BPW;
    for (int j = 0; j < GR_BPW; j++) {
        const uint64_t b = b0 + j;
        if (b >= nblocks) break;
        const int r = rbs[b];
        const uint64_t i = b * 32 + lane;
        if (r < e) {
            uint32_t w = 0, sg = 0;
            if (src && lane >= r) {
                if (lane == r) { sg = src[off0]; w = src[off0 + 1]; }
                else w = src[off0];
            }
            uint32_t sign;
            if (r >= s) {
                sign = __shfl_sync(FULL, sg, r);
                if (signs && lane == 0) signs[b] = sign;
            } else {
                sign = signs[b];
            }
            const uint32_t col = transpose32(w, lane);
            const uint32_t acc = __brev(col) >> (32 - e);
            const float v = scale2((float)acc, exp - e, fast, sc);
            if (i < n) out[i] = ((sign >> lane) & 1u) ? -v : v;
        } else {
            if (i < n) out[i] = 0.f;
        }
        off0 += gr_words(r, lane);
    }
}

// fp32 grouped pass 1: each block's recording bitplane and the chunk's word counts
__global__ void __launch_bounds__(256) k_gr_rb32(const float* __restrict__ x, uint64_t n,
                                                const uint32_t* __restrict__ maxkey, int exp_arg, int B,
                                                uint8_t* __restrict__ rbs, uint32_t* __restrict__ chunk_words) {
    const int exp = maxkey ? frexp_exp(__uint_as_float(*maxkey)) : exp_arg;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint64_t nblocks = (n + 31) / 32;
    __shared__ uint32_t cnt[GR_WARPS][32];
    uint32_t c0 = 0;
    const bool fast = pow2_normal(B - exp);
    const float sc = fast ? pow2f(B - exp) : 1.f;
    const uint64_t b0 = (uint64_t)blockIdx.x * GR_CHUNK + (uint64_t)warp * GR_BPW;
    for (int j = 0; j < GR_BPW; j++) {
        const uint64_t b = b0 + j;
        if (b >= nblocks) break;
        const uint64_t i = b * 32 + lane;
        uint32_t q = 0;
        if (i < n) {
            const float sh = scale2(__ldg(x + i), B - exp, fast, sc);
            const int64_t fix = (int64_t)sh;
            q = (uint32_t)(fix < 0 ? -fix : fix);
        }
        const uint32_t o = __reduce_or_sync(FULL, q);
        const int r = o ? B - 1 - (31 - __clz(o)) : B;
        if (lane == 0) rbs[b] = (uint8_t)r;
        c0 += gr_words(r, lane);
    }
    cnt[warp][lane] = c0;
    __syncthreads();
    if (threadIdx.x < 32 && (int)threadIdx.x < B) {
        uint32_t t = 0;
        for (int w = 0; w < GR_WARPS; w++) t += cnt[w][threadIdx.x];
        chunk_words[(uint64_t)blockIdx.x * B + threadIdx.x] = t;
    }
}

// GroupedBPEncoder::progressive_decode -- :210-297 (planes [s, e)); plane p's
// words at planes[p] (absolute plane index). signs: per-block sign words kept
// between calls (nullable when s == 0). A device count (dnum[0]) overrides e.
template <class T>
__global__ void __launch_bounds__(256) k_gr_decode(const typename Traits<T>::S* const* __restrict__ planes,
                                                   uint64_t n, const typename KeyOf<T>::type* __restrict__ maxkey,
                                                   int exp_arg, int B, int s, int e,
                                                   const uint8_t* __restrict__ dnum, const uint8_t* __restrict__ rbs,
                                                   const uint32_t* __restrict__ chunk_off,
                                                   typename Traits<T>::S* __restrict__ signs, T* __restrict__ out) {
    using S = typename Traits<T>::S;
    using FP = typename Traits<T>::FP;
    constexpr int BS = Traits<T>::kBlock;
    if (dnum) e = dnum[0];
    const int exp = level_exp<T>(maxkey, exp_arg);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint64_t nblocks = (n + BS - 1) / BS;
    uint32_t off0, off1;
    gr_warp_offsets(rbs, nblocks, chunk_off, B, off0, off1);
    const uint64_t b0 = (uint64_t)blockIdx.x * GR_CHUNK + (uint64_t)warp * GR_BPW;
    for (int j = 0; j < GR_BPW; j++) {
        uint64_t b = b0 + j;
        if (b >= nblocks) break;
        const int r = rbs[b];
        if (r < e) {
            S w0 = 0, w1 = 0, sg0 = 0, sg1 = 0;
            int p0 = lane, p1 = lane + 32;
            if (p0 < e && p0 >= s && p0 >= r) {
                const S* src = planes[p0] + off0;
                if (p0 == r) { sg0 = src[0]; w0 = src[1]; } else w0 = src[0];
            }
            if (p1 < e && p1 >= s && p1 >= r) {
                const S* src = planes[p1] + off1;
                if (p1 == r) { sg1 = src[0]; w1 = src[1]; } else w1 = src[0];
            }
            S sign;
            if (r >= s) {
                sign = __shfl_sync(FULL, r < 32 ? sg0 : sg1, r & 31);
                if (signs && lane == 0) signs[b] = sign;
            } else {
                sign = signs[b];
            }
            FP acc[BS / 32];
#pragma unroll
            for (int h = 0; h < BS / 32; h++) acc[h] = 0;
            if constexpr (BS == 64) {
                // decode_block :359-368 by four warp bit transposes: lane p holds
                // planes p and p + 32 (zero where not read); after the
                // transposes lane v holds, per half h of the block, a word whose
                // bit p is plane p's bit of value 32 h + v (planes 0..31) and one
                // for planes 32..63. Plane p weighs 2^(e-1-p): the bit-reversed
                // words, shifted into place.
                const uint32_t pl0 = transpose32((uint32_t)w0, lane), ph0 = transpose32((uint32_t)(w0 >> 32), lane);
                const uint32_t pl1 = transpose32((uint32_t)w1, lane), ph1 = transpose32((uint32_t)(w1 >> 32), lane);
                const uint32_t lo[2] = {pl0, ph0}, hi[2] = {pl1, ph1};
#pragma unroll
                for (int h = 0; h < 2; h++) {
                    // planes 0..31 -> bits e-1 .. e-32, planes 32..63 -> bits e-33 ..
                    const uint64_t a = (uint64_t)__brev(lo[h]) << 32 | __brev(hi[h]);   // plane p at bit 63 - p
                    acc[h] = (FP)(e > 0 ? a >> (64 - e) : 0ull);
                }
            } else {
                const int first = r > s ? r : s;
                for (int p = first; p < e; p++) {             // decode_block :359-368
                    S w = __shfl_sync(FULL, p < 32 ? w0 : w1, p & 31);
                    const int k = e - 1 - p;
#pragma unroll
                    for (int h = 0; h < BS / 32; h++) acc[h] |= (FP)((w >> (h * 32 + lane)) & 1u) << k;
                }
            }
#pragma unroll
            for (int h = 0; h < BS / 32; h++) {
                uint64_t i = b * BS + h * 32 + lane;
                if (i < n) out[i] = gr_value<T>(acc[h], -e + exp, (sign >> (h * 32 + lane)) & 1u);
            }
        } else {
#pragma unroll
            for (int h = 0; h < BS / 32; h++) {
                uint64_t i = b * BS + h * 32 + lane;
                if (i < n) out[i] = (T)0;
            }
        }
        off0 += gr_words(r, lane);
        off1 += gr_words(r, lane + 32);
    }
}

// ---------------------------------------------------------------------------
// Squared error collector -- SquaredErrorCollector.hpp:54-96. The bit-clearing
// loop is evaluated in closed form: entry k receives (v - v with bits <= b
// cleared)^2 for b = exp_diff + (idx0 - k) while b < prec, else v^2.
// ---------------------------------------------------------------------------
template <class T>
__global__ void __launch_bounds__(256) k_sq_collect(const T* __restrict__ x, uint64_t n, int B, T maxv,
                                                    double* __restrict__ partial) {
    using A = typename Acc<T>::type;
    using U = typename Traits<T>::Bits;
    constexpr int prec = Traits<T>::kPrec;
    A acc[Acc<T>::N];
#pragma unroll
    for (int k = 0; k < Acc<T>::N; k++) acc[k] = 0;
    const int lexp = frexp_exp(maxv);
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        T v = x[i];
        if (v == (T)0) continue;
        int de = frexp_exp(v);
        U bits;
        memcpy(&bits, &v, sizeof(T));
        int exp_diff = lexp - de + prec - B;
        int idx0 = B;
        if (exp_diff <= 0) { idx0 += exp_diff; exp_diff = 0; }
        if (idx0 <= 0) continue;
        const T vv = v * v;
#pragma unroll
        for (int k = 0; k < Acc<T>::N; k++) {
            if (k <= idx0 && k <= B) {
                int bb = exp_diff + (idx0 - k);
                if (bb < prec) {
                    U cleared = bits & ~((((U)2) << bb) - (U)1);
                    T f;
                    memcpy(&f, &cleared, sizeof(T));
                    T d = v - f;
                    acc[k] += (A)(d * d);
                } else {
                    acc[k] += (A)vv;
                }
            }
        }
    }
    flush_errors(acc, B, partial);
}

// sum partial tables in fixed order, then scale by 2^(2*(exp - B)) when exp
// scaling applies (encoder tables, NegaBinaryBPEncoder.hpp:121-123).
template <class T>
__global__ void k_reduce_partials(const double* __restrict__ partial, int nparts, int B,
                                  const typename KeyOf<T>::type* __restrict__ maxkey, int exp_arg, int exp_add,
                                  int scale, double* __restrict__ out) {
    // one warp per table entry; lane-strided partial sums then a fixed-order
    // shuffle tree, so the result does not depend on scheduling
    const int lane = threadIdx.x & 31;
    for (int k = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); k <= B; k += gridDim.x * (blockDim.x >> 5)) {
        double s = 0;
        for (int p = lane; p < nparts; p += 32) s += partial[(size_t)p * (B + 1) + k];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(FULL, s, o);
        if (lane == 0) {
            if (scale) {
                int exp = level_exp<T>(maxkey, exp_arg) + exp_add;
                s = ldexp(s, 2 * (-B + exp));
            }
            out[k] = s;
        }
    }
}

// MaxErrorCollector::collect_level_error -- MaxErrorCollector.hpp:14-25, for
// all levels at once from the device bound array.
template <class T>
__global__ void k_max_collect(const T* __restrict__ bounds, int nl, int B, double* __restrict__ out) {
    for (int l = blockIdx.x * blockDim.x + threadIdx.x; l < nl; l += gridDim.x * blockDim.x) {
        T bound = bounds[l];
        int e = frexp_exp(bound);
        double* o = out + (size_t)l * (B + 1);
        o[0] = (double)bound;
        double err = ldexp(1.0, e - 1);
        for (int i = 1; i <= B; i++) { o[i] = err; err /= 2; }
    }
}

// per-chunk word counts from an rb array (used when only the header is known)
__global__ void k_chunk_words_from_rb(const uint8_t* __restrict__ rbs, uint64_t nblocks, int B,
                                      uint32_t* __restrict__ chunk_words) {
    __shared__ uint32_t cnt[GR_WARPS][64];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint64_t b0 = (uint64_t)blockIdx.x * GR_CHUNK + (uint64_t)warp * GR_BPW;
    uint32_t c0 = 0, c1 = 0;
    for (int j = 0; j < GR_BPW; j++) {
        uint64_t b = b0 + j;
        if (b >= nblocks) break;
        int r = rbs[b];
        c0 += gr_words(r, lane);
        c1 += gr_words(r, lane + 32);
    }
    cnt[warp][lane] = c0;
    cnt[warp][lane + 32] = c1;
    __syncthreads();
    if (threadIdx.x < 64 && (int)threadIdx.x < B) {
        uint32_t s = 0;
        for (int w = 0; w < GR_WARPS; w++) s += cnt[w][threadIdx.x];
        chunk_words[(uint64_t)blockIdx.x * B + threadIdx.x] = s;
    }
}

}  // namespace

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
// opt-in to more than 48 KB of dynamic shared memory, once per device and kernel
static int allow_smem(const void* k, size_t bytes) {
    static std::mutex mu;
    static std::vector<std::pair<int, const void*>> done;
    int dev = 0;
    PRODM_CUDA(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lock(mu);
    for (const auto& d : done)
        if (d.first == dev && d.second == k) return PRODM_OK;
    PRODM_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
    done.push_back({dev, k});
    return PRODM_OK;
}

// the opt-in comes first: the occupancy query counts it
static unsigned nb_err_grid(uint64_t need) {
    (void)allow_smem((const void*)k_nb_encode32_err, kErrSmemNB);
    return persistent_grid_for((const void*)k_nb_encode32_err, 256, kErrSmemNB, need, kPartialSlots);
}

// fp32 negabinary with tables: the encode launch (records in partial), then
// the final reduction of nseg levels into errs_out
static int nb_err_launch(const ChunkSeg* segs, const ChunkSeg& one, int nseg, uint64_t total, int B, int exp,
                         double* partial, double* errs_out, cudaStream_t st) {
    int rc;
    if ((rc = allow_smem((const void*)k_nb_encode32_err, kErrSmemNB))) return rc;
    const unsigned grid = nb_err_grid(segs ? (uint64_t)kPartialSlots : total);
    unsigned long long* recs = (unsigned long long*)partial;
    k_nb_encode32_err<<<grid, 256, kErrSmemNB, st>>>(segs, one, nseg, total, B, exp, recs);
    PRODM_CHECK_LAUNCH("k_nb_encode32_err");
    k_errtab_final<true><<<nseg, 1024, 0, st>>>(recs, (int)grid, B, segs, one, exp, 2, errs_out);
    PRODM_CHECK_LAUNCH("k_errtab_final");
    return PRODM_OK;
}

template <class T>
int launch_nb_encode(const T* x, uint64_t n, const void* maxkey, int exp, int B, void* out, uint64_t stride,
                     double* partial, double* errs_out, cudaStream_t st) {
    using K = typename KeyOf<T>::type;
    constexpr int BS = Traits<T>::kBlock;
    const uint64_t nblocks = (n + BS - 1) / BS;
    const int th = 256;
    if (std::is_same<T, float>::value) {
        const uint64_t nch = (nblocks + NB_CHUNK - 1) / NB_CHUNK;
        if (errs_out) {
            ChunkSeg one = {};
            one.x = (const float*)x;
            one.words = (uint32_t*)out;
            one.n = n;
            one.nblocks = nblocks;
            one.stride = stride;
            one.key = (const uint32_t*)maxkey;
            return nb_err_launch(nullptr, one, 1, nch, B, exp, partial, errs_out, st);
        }
        const unsigned grid = persistent_grid_for((const void*)k_nb_encode32, th, 0, nch, nch);
        k_nb_encode32<<<grid, th, 0, st>>>((const float*)x, n, (const uint32_t*)maxkey, exp, B, (uint32_t*)out, stride);
        PRODM_CHECK_LAUNCH("k_nb_encode32");
        return PRODM_OK;
    }
    const unsigned grid = errs_out ? persistent_grid_for((const void*)k_nb_encode<T, true>, th, 0, nblocks, kPartialSlots)
                                   : grid_for(nblocks * 32, th, 8);
    if (errs_out) {
        k_nb_encode<T, true><<<grid, th, 0, st>>>(x, n, (const K*)maxkey, exp, B, (typename Traits<T>::S*)out, stride,
                                                  partial);
        PRODM_CHECK_LAUNCH("k_nb_encode");
        k_reduce_partials<T><<<(B + 8) / 8, 256, 0, st>>>(partial, (int)grid, B, (const K*)maxkey, exp, 2, 1, errs_out);
        PRODM_CHECK_LAUNCH("k_reduce_partials");
    } else {
        k_nb_encode<T, false><<<grid, th, 0, st>>>(x, n, (const K*)maxkey, exp, B, (typename Traits<T>::S*)out, stride,
                                                   nullptr);
        PRODM_CHECK_LAUNCH("k_nb_encode");
    }
    return PRODM_OK;
}

int launch_nb_decode_levels(const ChunkSeg* segs, int nseg, uint64_t total_chunks, cudaStream_t st, bool pdl) {
    const unsigned grid = persistent_grid_for((const void*)k_nb_decode_levels, 256, 0, total_chunks, total_chunks);
    count_launch();
    const cudaError_t e = launch_chain(pdl, k_nb_decode_levels, dim3(grid), dim3(256), 0, st, segs, nseg, total_chunks);
    if (e != cudaSuccess) return cuda_status(e, "k_nb_decode_levels");
    return PRODM_OK;
}

int nb_encode_levels_grid(int with_errors) {
    if (with_errors) return (int)nb_err_grid((uint64_t)kPartialSlots);
    return (int)persistent_grid_for((const void*)k_nb_encode32_levels, 256, 0, (uint64_t)kPartialSlots, kPartialSlots);
}

int launch_nb_encode_levels(const ChunkSeg* segs, int nseg, uint64_t total_chunks, int B, double* partial,
                            const uint32_t* keys, double* errs_out, cudaStream_t st) {
    (void)keys;   // each segment carries its level's key
    if (errs_out) return nb_err_launch(segs, ChunkSeg{}, nseg, total_chunks, B, 0, partial, errs_out, st);
    const unsigned grid = (unsigned)nb_encode_levels_grid(0);
    k_nb_encode32_levels<<<grid, 256, 0, st>>>(segs, nseg, total_chunks, B);
    PRODM_CHECK_LAUNCH("k_nb_encode32_levels");
    return PRODM_OK;
}

template <class T>
int launch_nb_decode(const void* base, uint64_t stride, uint64_t n, const void* maxkey, int exp, int s, int num,
                     const uint8_t* dnum, T* out, cudaStream_t st) {
    using K = typename KeyOf<T>::type;
    constexpr int BS = Traits<T>::kBlock;
    const uint64_t nblocks = (n + BS - 1) / BS;
    const int th = 256;
    if (std::is_same<T, float>::value) {
        const uint64_t nch = (nblocks + NB_CHUNK - 1) / NB_CHUNK;
        const unsigned grid = persistent_grid_for((const void*)k_nb_decode32, th, 0, nch, nch);
        k_nb_decode32<<<grid, th, 0, st>>>((const uint32_t*)base, stride, n, (const uint32_t*)maxkey, exp, s, num, dnum,
                                           (float*)out);
        PRODM_CHECK_LAUNCH("k_nb_decode32");
        return PRODM_OK;
    }
    k_nb_decode<T><<<grid_for(nblocks * 32, th, 8), th, 0, st>>>((const typename Traits<T>::S*)base, stride, n,
                                                                 (const K*)maxkey, exp, s, num, dnum, out);
    PRODM_CHECK_LAUNCH("k_nb_decode");
    return PRODM_OK;
}

uint64_t gr_nchunks(uint64_t nblocks) { return (nblocks + GR_CHUNK - 1) / GR_CHUNK; }

template <class T>
int launch_gr_encode(const T* x, uint64_t n, const void* maxkey, int exp, int B, uint8_t* rbs, uint32_t* chunk_words,
                     uint32_t* chunk_off, uint32_t* sizes, void* out, uint64_t cap, double* partial, double* errs_out,
                     cudaStream_t st) {
    using K = typename KeyOf<T>::type;
    constexpr int BS = Traits<T>::kBlock;
    const uint64_t nblocks = (n + BS - 1) / BS;
    const uint64_t nch = gr_nchunks(nblocks);
    if (std::is_same<T, float>::value) {
        k_gr_rb32<<<(unsigned)nch, GR_WARPS * 32, 0, st>>>((const float*)x, n, (const uint32_t*)maxkey, exp, B, rbs,
                                                          chunk_words);
        PRODM_CHECK_LAUNCH("k_gr_rb32");
        k_gr_scan<<<B, 1024, 0, st>>>(chunk_words, nch, B, nblocks, 4, chunk_off, sizes);
        PRODM_CHECK_LAUNCH("k_gr_scan");
        unsigned long long* recs = (unsigned long long*)partial;
        if (errs_out) {
            k_gr_write32<true><<<(unsigned)nch, GR_WARPS * 32, kErrSmemGR, st>>>(
                (const float*)x, n, (const uint32_t*)maxkey, exp, B, rbs, chunk_off, (uint32_t*)out, cap, recs);
            PRODM_CHECK_LAUNCH("k_gr_write32");
            ChunkSeg one = {};
            one.n = n;
            one.key = (const uint32_t*)maxkey;
            k_errtab_final<false><<<1, 1024, 0, st>>>(recs, (int)nch, B, nullptr, one, exp, 0, errs_out);
            PRODM_CHECK_LAUNCH("k_errtab_final");
        } else {
            k_gr_write32<false><<<(unsigned)nch, GR_WARPS * 32, 0, st>>>(
                (const float*)x, n, (const uint32_t*)maxkey, exp, B, rbs, chunk_off, (uint32_t*)out, cap, nullptr);
            PRODM_CHECK_LAUNCH("k_gr_write32");
        }
        return PRODM_OK;
    }
    if (errs_out) {
        k_gr_rb<T, true><<<(unsigned)nch, GR_WARPS * 32, 0, st>>>(x, n, (const K*)maxkey, exp, B, rbs, chunk_words,
                                                                  partial);
    } else {
        k_gr_rb<T, false><<<(unsigned)nch, GR_WARPS * 32, 0, st>>>(x, n, (const K*)maxkey, exp, B, rbs, chunk_words,
                                                                   nullptr);
    }
    PRODM_CHECK_LAUNCH("k_gr_rb");
    if (errs_out) {
        k_reduce_partials<T><<<(B + 8) / 8, 256, 0, st>>>(partial, (int)nch, B, (const K*)maxkey, exp, 0, 1, errs_out);
        PRODM_CHECK_LAUNCH("k_reduce_partials");
    }
    k_gr_scan<<<B, 1024, 0, st>>>(chunk_words, nch, B, nblocks, (int)sizeof(typename Traits<T>::S), chunk_off, sizes);
    PRODM_CHECK_LAUNCH("k_gr_scan");
    k_gr_write<T><<<(unsigned)nch, GR_WARPS * 32, 0, st>>>(x, n, (const K*)maxkey, exp, B, rbs, chunk_off,
                                                           (typename Traits<T>::S*)out, cap);
    PRODM_CHECK_LAUNCH("k_gr_write");
    return PRODM_OK;
}

int launch_chunk_words_from_rb(const uint8_t* rbs, uint64_t nblocks, int B, uint32_t* chunk_words, cudaStream_t st) {
    const uint64_t nch = gr_nchunks(nblocks);
    k_chunk_words_from_rb<<<(unsigned)nch, GR_WARPS * 32, 0, st>>>(rbs, nblocks, B, chunk_words);
    PRODM_CHECK_LAUNCH("k_chunk_words_from_rb");
    return PRODM_OK;
}

int launch_gr_scan_only(const uint32_t* chunk_words, uint64_t nchunks, int B, uint64_t nblocks, int word_bytes,
                        uint32_t* chunk_off, uint32_t* sizes, cudaStream_t st) {
    k_gr_scan<<<B, 1024, 0, st>>>(chunk_words, nchunks, B, nblocks, word_bytes, chunk_off, sizes);
    PRODM_CHECK_LAUNCH("k_gr_scan");
    return PRODM_OK;
}

template <class T>
int launch_gr_decode(const void* const* planes, uint64_t n, const void* maxkey, int exp, int B, int s, int e,
                     const uint8_t* dnum, const uint8_t* rbs, const uint32_t* chunk_off, void* signs, T* out,
                     cudaStream_t st) {
    using K = typename KeyOf<T>::type;
    using S = typename Traits<T>::S;
    constexpr int BS = Traits<T>::kBlock;
    const uint64_t nblocks = (n + BS - 1) / BS;
    const uint64_t nch = gr_nchunks(nblocks);
    if (std::is_same<T, float>::value) {
        k_gr_decode32<<<(unsigned)nch, GR_WARPS * 32, 0, st>>>((const uint32_t* const*)planes, n,
                                                              (const uint32_t*)maxkey, exp, B, s, e, dnum, rbs,
                                                              chunk_off, (uint32_t*)signs, (float*)out);
        PRODM_CHECK_LAUNCH("k_gr_decode32");
        return PRODM_OK;
    }
    k_gr_decode<T><<<(unsigned)nch, GR_WARPS * 32, 0, st>>>((const S* const*)planes, n, (const K*)maxkey, exp, B, s, e,
                                                            dnum, rbs, chunk_off, (S*)signs, out);
    PRODM_CHECK_LAUNCH("k_gr_decode");
    return PRODM_OK;
}

template <class T>
int launch_sq_collect(const T* x, uint64_t n, int B, T maxv, double* partial, double* out, cudaStream_t st) {
    const int th = 256;
    const unsigned grid = persistent_grid_for((const void*)k_sq_collect<T>, th, 0, (n + th - 1) / th, kPartialSlots);
    k_sq_collect<T><<<grid, th, 0, st>>>(x, n, B, maxv, partial);
    PRODM_CHECK_LAUNCH("k_sq_collect");
    k_reduce_partials<T><<<(B + 8) / 8, 256, 0, st>>>(partial, (int)grid, B, nullptr, 0, 0, 0, out);
    PRODM_CHECK_LAUNCH("k_reduce_partials");
    return PRODM_OK;
}

template <class T>
int launch_max_collect(const T* bounds, int nl, int B, double* out, cudaStream_t st) {
    k_max_collect<T><<<1, 32, 0, st>>>(bounds, nl, B, out);
    PRODM_CHECK_LAUNCH("k_max_collect");
    return PRODM_OK;
}

#define INST(T)                                                                                                       \
    template int launch_nb_encode<T>(const T*, uint64_t, const void*, int, int, void*, uint64_t, double*, double*,    \
                                     cudaStream_t);                                                                   \
    template int launch_nb_decode<T>(const void*, uint64_t, uint64_t, const void*, int, int, int, const uint8_t*, T*, \
                                     cudaStream_t);                                                                   \
    template int launch_gr_encode<T>(const T*, uint64_t, const void*, int, int, uint8_t*, uint32_t*, uint32_t*,       \
                                     uint32_t*, void*, uint64_t, double*, double*, cudaStream_t);                     \
    template int launch_gr_decode<T>(const void* const*, uint64_t, const void*, int, int, int, int, const uint8_t*,   \
                                     const uint8_t*, const uint32_t*, void*, T*, cudaStream_t);                       \
    template int launch_sq_collect<T>(const T*, uint64_t, int, T, double*, double*, cudaStream_t);                   \
    template int launch_max_collect<T>(const T*, int, int, double*, cudaStream_t);
INST(float)
INST(double)
#undef INST

}  // namespace prodm
