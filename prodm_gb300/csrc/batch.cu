// Batched refactor / retrieve of many fields of different shapes (sm_103a).
//
// Every stage runs as one persistent launch over all fields: a device table
// of segments -- one per (field, level) -- maps each global row or chunk to
// its field, so the 64-field batch costs one launch per decomposition depth,
// one encode launch, one interpreter launch, one decode launch and one
// launch per recomposition depth, instead of one launch per level per field.
// No stage waits on another inside a kernel: the ordering between depths is
// the stream order (or the dependency edges of a captured CUDA graph).
// Fields share the bitplane count, encoder (negabinary), dtype (fp32) and
// basis (hierarchical); shapes and level counts are per field.
#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "common.cuh"
#include "kernels.cuh"
#include "nbcodec.cuh"
#include "rows.cuh"

namespace prodm {
// Fused finest levels with rows of 257 values and up whose 11-row units fit
// a 96-word box take the warp-specialised batched kernel (64-field batch,
// same launch shapes: 2.60 ms per step against 2.73 ms with the 8-warp
// kernel). PRODM_BATCH_WS=0 keeps them on the 8-warp kernel; read when a
// batch is planned.
static bool batch_ws() {
    const char* v = getenv("PRODM_BATCH_WS");
    return !v || atoi(v) != 0;
}
// shortest row (values) that takes the warp-specialised batched kernel;
// PRODM_BATCH_WS_MIN_ROW overrides 257 (64-field batch: 2.610 ms at 257,
// 2.620 ms at 129, 2.782 ms at 65, where units of 11 short rows are small)
static uint32_t batch_ws_min_row() {
    const char* v = getenv("PRODM_BATCH_WS_MIN_ROW");
    return v ? (uint32_t)atoi(v) : 257u;
}

namespace {

constexpr int kMaxL = 17;

struct RowSeg {
    Box F, C;
    const float* in;        // decompose: fine box; recompose: coarse box
    float* coef;            // level coefficients (packed)
    float* out;             // decompose: coarse box; recompose: fine box
    uint64_t s0, s1;        // strides of the fine box (decompose input / recompose output)
    uint32_t row_begin;
    uint32_t* key_l;        // decompose: level |max| key
    uint32_t* key_c;        // decompose at level 1: level-0 |max| key
    uint32_t patch;         // work items are patch items (decompose_ / recompose_patch_item), not rows:
                            // every 2^k + 1 level of a batch (all fields' levels share one launch,
                            // so the single-field path's minimum item count does not apply)
};

// segment of global row g: binary search over the segments' first rows,
// staged in shared memory (one dependent shared load per step instead of a
// global one)
__device__ __forceinline__ int find_row_seg(const uint32_t* begins, int nseg, uint32_t g) {
    int lo = 0, hi = nseg - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (begins[mid] <= g) lo = mid; else hi = mid - 1;
    }
    return lo;
}
__device__ __forceinline__ void stage_row_begins(const RowSeg* segs, int nseg, uint32_t* begins) {
    for (int i = threadIdx.x; i < nseg; i += blockDim.x) begins[i] = segs[i].row_begin;
    __syncthreads();
}

__global__ void __launch_bounds__(256, 3) k_decompose_multi(const RowSeg* __restrict__ segs, int nseg, uint32_t total) {
    extern __shared__ uint32_t s_begin[];
    stage_row_begins(segs, nseg, s_begin);
    const uint32_t lane = threadIdx.x & 31, wpb = blockDim.x >> 5;
    uint32_t mk = 0, mc = 0;
    int cur = -1;
    auto flush = [&]() {
        if (cur < 0) return;
        uint32_t a = warp_max_key(mk), b = warp_max_key(mc);
        if (lane == 0) {
            if (a) atomicMax(segs[cur].key_l, a);
            if (b && segs[cur].key_c) atomicMax(segs[cur].key_c, b);
        }
        mk = mc = 0;
    };
    for (uint32_t g = blockIdx.x * wpb + (threadIdx.x >> 5); g < total; g += gridDim.x * wpb) {
        const int s = find_row_seg(s_begin, nseg, g);
        if (s != cur) { flush(); cur = s; }
        const RowSeg& q = segs[s];
        if (q.patch)
            decompose_patch_item<float>(q.in, q.s0, q.s1, q.F, q.C, q.coef, q.out, g - q.row_begin, lane, mk, mc);
        else if (q.F.n[2] & 1u)
            decompose_row_odd_any<float>(q.in, q.s0, q.s1, q.F, q.C, q.coef, q.out, nullptr, g - q.row_begin, lane,
                                         mk, mc);
        else
            decompose_row<float>(q.in, q.s0, q.s1, q.F, q.C, q.coef, q.out, nullptr, g - q.row_begin, lane, mk, mc);
    }
    flush();
}

__global__ void __launch_bounds__(256) k_recompose_multi(const RowSeg* __restrict__ segs, int nseg, uint32_t total) {
    extern __shared__ uint32_t s_begin[];
    stage_row_begins(segs, nseg, s_begin);
    const uint32_t lane = threadIdx.x & 31, wpb = blockDim.x >> 5;
    for (uint32_t g = blockIdx.x * wpb + (threadIdx.x >> 5); g < total; g += gridDim.x * wpb) {
        const int s = find_row_seg(s_begin, nseg, g);
        const RowSeg& q = segs[s];
        if (q.patch)
            recompose_patch_item<float>(q.in, q.coef, q.F, q.C, q.out, q.s0, q.s1, g - q.row_begin, lane);
        else if (q.F.n[2] & 1u)
            recompose_row_odd_any<float>(q.in, q.coef, q.F, q.C, q.out, q.s0, q.s1, g - q.row_begin, lane);
        else
            recompose_row<float>(q.in, q.coef, q.F, q.C, q.out, q.s0, q.s1, g - q.row_begin, lane);
    }
}

__global__ void __launch_bounds__(256) k_nb_encode_multi(const ChunkSeg* __restrict__ segs, int nseg, uint64_t total,
                                                        int B) {
    __shared__ uint32_t tile[32 * NB_TILE_LD];
    for (uint64_t c = blockIdx.x; c < total; c += gridDim.x) {
        const int s = find_seg(segs, nseg, c, &ChunkSeg::chunk_begin);
        const ChunkSeg& q = segs[s];
        const int exp = frexp_exp(__uint_as_float(*q.key)) + 2;     // NegaBinaryBPEncoder.hpp:21
        const int se = B - exp;
        const bool fast = pow2_normal(se);
        nb_encode32_chunk(q.x, q.n, q.nblocks, B, se, fast, fast ? pow2f(se) : 1.f, q.words, q.stride,
                          c - q.chunk_begin, tile);
    }
}

// per (field, level) slot: bound = 4 |max| (negabinary) and the max-error
// table (MaxErrorCollector.hpp:14-25)
__global__ void k_bounds_tables_multi(const uint32_t* __restrict__ keys, const int* __restrict__ levels, int nf, int B,
                                      float* __restrict__ bounds, double* __restrict__ maxerr) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nf * kMaxL) return;
    const int f = i / kMaxL, l = i - f * kMaxL;
    if (l > levels[f]) return;
    const float b = __uint_as_float(keys[i]) * 4.f;
    bounds[i] = b;
    double* o = maxerr + (size_t)i * (B + 1);
    int e;
    frexpf(b, &e);
    o[0] = (double)b;
    double err = ldexp(1.0, e - 1);
    for (int k = 1; k <= B; k++) { o[k] = err; err /= 2; }
}

}  // namespace
}  // namespace prodm

using namespace prodm;

struct prodm_batch {
    int nf = 0, B = 0;
    std::vector<prodm_config> cfg;
    std::vector<LevelGeom> g;
    std::vector<void*> allocs;
    // per field offsets into the arenas (elements / bytes)
    std::vector<uint64_t> coef_off, rcoef_off, cb_off, cb_len, stream_off;
    std::vector<std::vector<uint64_t>> roff;       // decoded level offsets within a field (16-byte aligned)
    std::vector<std::vector<uint64_t>> lvl_stream_off;
    float* coef = nullptr;
    float* rcoef = nullptr;
    float* cbuf = nullptr;    // 2 * cb_len per field
    float* rbuf = nullptr;
    uint8_t* streams = nullptr;
    uint32_t* keys = nullptr;     // [nf][17]
    float* bounds = nullptr;      // [nf][17]
    uint32_t* sizes = nullptr;    // [nf][17][B]
    double* maxerr = nullptr;     // [nf][17][B+1]
    uint8_t* index = nullptr;     // [nf][17]
    uint32_t* rsz = nullptr;
    int* ndims_d = nullptr;
    int* levels_d = nullptr;
    double* tols = nullptr;
    int maxL = 0;
    // segment tables (device) and their sizes
    std::vector<RowSeg*> dseg, rseg;
    std::vector<int> dn, rn;
    std::vector<uint32_t> drows, rrows;
    ChunkSeg* eseg = nullptr;
    ChunkSeg* decseg = nullptr;                    // decode: kDecodeChunkBlocks blocks per chunk
    int en = 0, decn = 0;
    uint64_t echunks = 0, dchunks = 0;
    // finest levels decoded inside their recomposition: fields whose plane
    // runs fit a TMA box of at most 96 words (fseg[0]) or 160 words (fseg[1])
    // (tensor maps in fmaps, one per field), fields with longer rows
    // (fseg[2]: cp.async staging), and fields with rows of 257 values and up
    // whose 11-row units fit a 96-word tall box (fseg[3]: the
    // warp-specialised batched kernel; before the other classes)
    FusedSeg* fseg[4] = {nullptr, nullptr, nullptr, nullptr};
    int fn[4] = {0, 0, 0, 0};
    uint64_t funits[4] = {0, 0, 0, 0};
    uint32_t ftld[4] = {0, 0, 0, 0};
    uint32_t fbw[4] = {0, 0, 0, 0};                // widest TMA box of each class
    uint8_t* fmaps = nullptr;                      // [nf][128] tensor maps
    int* kstatus = nullptr;                        // status word of the fused kernels
    std::vector<char> fused;                       // per field
    std::vector<const float*> fields;
    std::vector<float*> outs;
    bool bound = false;
    // launch shape per stage (decompose, encode, recompose): threads per CTA,
    // CTAs per SM of the persistent grid
    int st_threads[4] = {256, 256, 256, 256}, st_ctas[4] = {8, 8, 8, 0};
    // values per unit of the fused finest levels (TMA form): the tile shape
    // the autotuner searches with prodm_batch_set_fused_unit
    uint32_t unit_values = 2112;
    ~prodm_batch() {
        for (void* p : allocs) cudaFree(p);
    }
    int alloc(void** p, size_t bytes) {
        cudaError_t e = cudaMalloc(p, bytes ? bytes : 256);
        if (e != cudaSuccess) return cuda_status(e, "cudaMalloc");
        allocs.push_back(*p);
        return PRODM_OK;
    }
};

namespace prodm {
namespace {

// a field's finest level is fused when its rows have odd length and an
// 8-row unit's tiles fit the fused kernel's shared memory
bool batch_field_fused(const LevelGeom& g) {
    if (g.L < 1) return false;
    const Box& F = g.box[g.L];
    return (F.n[2] & 1u) && fused_multi_smem(fused_unit_blocks(F)) <= 200 * 1024;
}

int batch_build_segments(prodm_batch* h) {
    const int nf = h->nf, B = h->B;
    int rc;
    h->fused.assign(nf, 0);
    for (int f = 0; f < nf; f++) h->fused[f] = batch_field_fused(h->g[f]) ? 1 : 0;
    // decompose depths: depth d processes level L_f - d of every field with L_f - d >= 1
    h->dseg.assign(h->maxL, nullptr);
    h->rseg.assign(h->maxL, nullptr);
    h->dn.assign(h->maxL, 0);
    h->rn.assign(h->maxL, 0);
    h->drows.assign(h->maxL, 0);
    h->rrows.assign(h->maxL, 0);
    for (int d = 0; d < h->maxL; d++) {
        std::vector<RowSeg> ds, rs;
        uint32_t drow = 0, rrow = 0;
        for (int f = 0; f < nf; f++) {
            const LevelGeom& g = h->g[f];
            const int L = g.L;
            float* cb0 = h->cbuf + h->cb_off[f];
            float* cb1 = cb0 + h->cb_len[f];
            float* rb0 = h->rbuf + h->cb_off[f];
            float* rb1 = rb0 + h->cb_len[f];
            float* coef = h->coef + h->coef_off[f];
            float* rcoef = h->rcoef + h->rcoef_off[f];
            const int l = L - d;                  // decompose level at this depth
            if (l >= 1) {
                RowSeg s{};
                s.F = g.box[l];
                s.C = g.box[l - 1];
                s.in = (l == L) ? h->fields[f] : ((l + 1) & 1 ? cb1 : cb0);
                s.coef = coef + g.offset[l];
                s.out = (l == 1) ? coef + g.offset[0] : (l & 1 ? cb1 : cb0);
                s.s0 = (uint64_t)s.F.n[1] * s.F.n[2];
                s.s1 = s.F.n[2];
                s.row_begin = drow;
                s.key_l = h->keys + f * kMaxL + l;
                s.key_c = l == 1 ? h->keys + f * kMaxL : nullptr;
                s.patch = patch_grid(s.F, s.C) ? 1u : 0u;
                drow += s.patch ? (uint32_t)patch_items(s.C) : s.F.n[0] * s.F.n[1];
                ds.push_back(s);
            }
            const int lr = d + 1;                 // recompose level at this depth
            if (lr <= L && !(lr == L && h->fused[f])) {
                RowSeg s{};
                s.F = g.box[lr];
                s.C = g.box[lr - 1];
                s.in = (lr == 1) ? rcoef + h->roff[f][0] : ((lr - 1) & 1 ? rb1 : rb0);
                s.coef = rcoef + h->roff[f][lr];
                s.out = (lr == L) ? h->outs[f] : (lr & 1 ? rb1 : rb0);
                s.s0 = (uint64_t)s.F.n[1] * s.F.n[2];
                s.s1 = s.F.n[2];
                s.row_begin = rrow;
                s.patch = patch_grid(s.F, s.C) ? 1u : 0u;
                rrow += s.patch ? (uint32_t)patch_items(s.C) : s.F.n[0] * s.F.n[1];
                rs.push_back(s);
            }
        }
        h->dn[d] = (int)ds.size();
        h->rn[d] = (int)rs.size();
        h->drows[d] = drow;
        h->rrows[d] = rrow;
        if (!ds.empty()) {
            if (!h->dseg[d] && (rc = h->alloc((void**)&h->dseg[d], nf * sizeof(RowSeg)))) return rc;
            PRODM_CUDA(cudaMemcpy(h->dseg[d], ds.data(), ds.size() * sizeof(RowSeg), cudaMemcpyHostToDevice));
        }
        if (!rs.empty()) {
            if (!h->rseg[d] && (rc = h->alloc((void**)&h->rseg[d], nf * sizeof(RowSeg)))) return rc;
            PRODM_CUDA(cudaMemcpy(h->rseg[d], rs.data(), rs.size() * sizeof(RowSeg), cudaMemcpyHostToDevice));
        }
    }
    // fused finest levels
    {
        std::vector<FusedSeg> fs[4];
        uint64_t units[4] = {0, 0, 0, 0};
        uint32_t tld[4] = {0, 0, 0, 0};
        std::vector<uint8_t> maps((size_t)nf * 128, 0);
        if (!h->fmaps && (rc = h->alloc((void**)&h->fmaps, (size_t)nf * 128))) return rc;
        for (int f = 0; f < nf; f++) {
            if (!h->fused[f]) continue;
            const LevelGeom& g = h->g[f];
            const int L = g.L;
            FusedSeg s{};
            s.F = g.box[L];
            s.C = g.box[L - 1];
            const uint64_t nbk = (g.elems[L] + 31) / 32;
            s.base = (const uint32_t*)(h->streams + h->lvl_stream_off[f][L]);
            s.stride = (nbk + 3) / 4 * 4;
            s.key = h->keys + f * kMaxL + L;
            s.dnum = h->index + f * kMaxL + L;
            float* rb0 = h->rbuf + h->cb_off[f];
            float* rb1 = rb0 + h->cb_len[f];
            s.coarse = (L == 1) ? h->rcoef + h->rcoef_off[f] + h->roff[f][0] : ((L - 1) & 1 ? rb1 : rb0);
            s.out = h->outs[f];
            s.s0 = (uint64_t)s.F.n[1] * s.F.n[2];
            s.s1 = s.F.n[2];
            uint32_t t = fused_unit_blocks(s.F);
            s.rpu = fused_unit_rows(s.F, h->unit_values);
            s.bw = fused_tma_box(s.F, s.rpu);
            int k = 2;
            void* m = maps.data() + (size_t)f * 128;
            const uint32_t wr = fused_ws_unit_rows();
            const uint32_t wbw = (fused_unit_blocks_rows(s.F, wr) + 3 + 3) & ~3u;
            if (batch_ws() && s.F.n[2] >= batch_ws_min_row() && B <= 32 && wbw <= kWsMultiStride &&
                encode_plane_map(m, s.base, nbk, B, s.stride, kWsMultiStride, 32) == PRODM_OK) {
                k = 3;
                s.tall = 1;
                s.bw = wbw;
                s.rpu = wr;
                s.map = h->fmaps + (size_t)f * 128;
                t = fused_unit_blocks_rows(s.F, wr);
            } else if ((s.tall = s.bw && fused_tma_tall() && B <= 32 &&
                                 encode_plane_map(m, s.base, nbk, B, s.stride, fused_tma_stride(s.bw), 32) ==
                                     PRODM_OK) ||
                       (s.bw && encode_plane_map(m, s.base, nbk, B, s.stride, s.bw) == PRODM_OK)) {
                k = s.bw <= 96 ? 0 : 1;
                s.map = h->fmaps + (size_t)f * 128;
                t = fused_unit_blocks_rows(s.F, s.rpu);
            } else {
                s.bw = 0;
                s.map = nullptr;
                s.rpu = 8;
            }
            s.unit_begin = units[k];
            units[k] += ((uint64_t)s.F.n[0] * s.F.n[1] + s.rpu - 1) / s.rpu;
            tld[k] = std::max(tld[k], t);
            fs[k].push_back(s);
            h->fbw[k] = std::max(h->fbw[k], s.bw);
        }
        PRODM_CUDA(cudaMemcpy(h->fmaps, maps.data(), maps.size(), cudaMemcpyHostToDevice));
        for (int k = 0; k < 4; k++) {
            h->fn[k] = (int)fs[k].size();
            h->funits[k] = units[k];
            h->ftld[k] = tld[k];
            if (fs[k].empty()) continue;
            if (!h->fseg[k] && (rc = h->alloc((void**)&h->fseg[k], nf * sizeof(FusedSeg)))) return rc;
            PRODM_CUDA(cudaMemcpy(h->fseg[k], fs[k].data(), fs[k].size() * sizeof(FusedSeg), cudaMemcpyHostToDevice));
        }
    }
    // encode / decode: every (field, level); the decode skips fused finest levels
    std::vector<ChunkSeg> es, dc;
    uint64_t ch = 0, dch = 0;
    for (int f = 0; f < nf; f++) {
        const LevelGeom& g = h->g[f];
        for (int l = 0; l <= g.L; l++) {
            ChunkSeg s{};
            s.n = g.elems[l];
            s.nblocks = (s.n + 31) / 32;
            s.stride = (s.nblocks + 3) / 4 * 4;   // plane rows on 16-byte boundaries
            s.words = (uint32_t*)(h->streams + h->lvl_stream_off[f][l]);
            s.key = h->keys + f * kMaxL + l;
            s.dnum = h->index + f * kMaxL + l;
            s.x = h->coef + h->coef_off[f] + g.offset[l];
            s.y = h->rcoef + h->rcoef_off[f] + h->roff[f][l];
            ChunkSeg d = s;
            s.chunk_begin = ch;
            ch += (s.nblocks + NB_CHUNK - 1) / NB_CHUNK;
            es.push_back(s);
            if (l == g.L && h->fused[f]) continue;
            d.chunk_begin = dch;
            dch += (d.nblocks + kDecodeChunkBlocks - 1) / kDecodeChunkBlocks;
            dc.push_back(d);
        }
    }
    h->en = (int)es.size();
    h->decn = (int)dc.size();
    h->echunks = ch;
    h->dchunks = dch;
    if (!h->eseg && (rc = h->alloc((void**)&h->eseg, es.size() * sizeof(ChunkSeg)))) return rc;
    PRODM_CUDA(cudaMemcpy(h->eseg, es.data(), es.size() * sizeof(ChunkSeg), cudaMemcpyHostToDevice));
    if (!h->decseg && (rc = h->alloc((void**)&h->decseg, es.size() * sizeof(ChunkSeg)))) return rc;
    if (!dc.empty())
        PRODM_CUDA(cudaMemcpy(h->decseg, dc.data(), dc.size() * sizeof(ChunkSeg), cudaMemcpyHostToDevice));
    (void)B;
    return PRODM_OK;
}

unsigned persistent_grid(const prodm_batch* h, int stage, uint64_t work_items, unsigned items_per_cta) {
    uint64_t need = (work_items + items_per_cta - 1) / items_per_cta;
    uint64_t cap = (uint64_t)device_sms() * h->st_ctas[stage];
    uint64_t g = need < cap ? need : cap;
    return (unsigned)(g ? g : 1);
}

int batch_refactor(prodm_batch* h, cudaStream_t st) {
    PRODM_CUDA(cudaMemsetAsync(h->keys, 0, (size_t)h->nf * kMaxL * 4, st));
    const unsigned th = (unsigned)h->st_threads[0];
    for (int f = 0; f < h->nf; f++)
        if (h->g[f].L == 0) {
            PRODM_CUDA(cudaMemcpyAsync(h->coef + h->coef_off[f], h->fields[f], h->g[f].total * 4, cudaMemcpyDeviceToDevice, st));
            int rc = launch_maxabs<float>(h->coef + h->coef_off[f], h->g[f].total, h->keys + f * kMaxL, st);
            if (rc) return rc;
        }
    for (int d = 0; d < h->maxL; d++) {
        if (!h->dn[d]) continue;
        k_decompose_multi<<<persistent_grid(h, 0, h->drows[d], th / 32), th, h->dn[d] * 4, st>>>(h->dseg[d], h->dn[d],
                                                                                                 h->drows[d]);
        PRODM_CHECK_LAUNCH("k_decompose_multi");
    }
    k_nb_encode_multi<<<persistent_grid(h, 1, h->echunks, 1), 256, 0, st>>>(h->eseg, h->en, h->echunks, h->B);
    PRODM_CHECK_LAUNCH("k_nb_encode_multi");
    k_bounds_tables_multi<<<(h->nf * kMaxL + 127) / 128, 128, 0, st>>>(h->keys, h->levels_d, h->nf, h->B, h->bounds,
                                                                        h->maxerr);
    PRODM_CHECK_LAUNCH("k_bounds_tables_multi");
    return PRODM_OK;
}

int batch_retrieve(prodm_batch* h, int interp, int est, double s, cudaStream_t st) {
    int rc;
    const unsigned th = (unsigned)h->st_threads[2];
    if ((rc = launch_interpret<float>(h->nf, interp, est, h->ndims_d, h->levels_d, s, h->B, h->sizes,
                                      (uint64_t)kMaxL * h->B, h->maxerr, (uint64_t)kMaxL * (h->B + 1), h->tols, 0.0,
                                      h->index, kMaxL, h->rsz, st)))
        return rc;
    if (h->dchunks && (rc = launch_nb_decode_levels(h->decseg, h->decn, h->dchunks, st))) return rc;
    for (int f = 0; f < h->nf; f++)
        if (h->g[f].L == 0)
            PRODM_CUDA(cudaMemcpyAsync(h->outs[f], h->rcoef + h->rcoef_off[f], h->g[f].total * 4, cudaMemcpyDeviceToDevice, st));
    for (int d = 0; d < h->maxL; d++) {
        if (!h->rn[d]) continue;
        k_recompose_multi<<<persistent_grid(h, 2, h->rrows[d], th / 32), th, h->rn[d] * 4, st>>>(h->rseg[d], h->rn[d],
                                                                                                 h->rrows[d]);
        PRODM_CHECK_LAUNCH("k_recompose_multi");
    }
    // the finest levels whose coarse boxes the depths above completed
    const unsigned fc = (unsigned)h->st_ctas[PRODM_BATCH_FUSED];
    for (int k = 0; k < 2; k++)
        if (h->fn[k] && (rc = launch_decode_recompose_nb32_tma_multi(h->fseg[k], h->fn[k], h->funits[k], h->ftld[k],
                                                                    h->fbw[k], fc, h->kstatus, st)))
            return rc;
    if (h->fn[2] && (rc = launch_decode_recompose_nb32_multi(h->fseg[2], h->fn[2], h->funits[2], h->ftld[2], fc, st)))
        return rc;
    if (h->fn[3] && (rc = launch_decode_recompose_nb32_ws_multi(h->fseg[3], h->fn[3], h->funits[3], h->ftld[3],
                                                                 h->kstatus, st)))
        return rc;
    return PRODM_OK;
}

}  // namespace


}  // namespace prodm

extern "C" {

int prodm_batch_create(prodm_batch** out, int nfields, const prodm_config* cfgs) {
    if (!out || !cfgs || nfields < 1) return fail(PRODM_EINVAL, "prodm_batch_create: bad arguments");
    if (nfields > 4096) return fail(PRODM_EINVAL, "prodm_batch_create: at most 4096 fields per batch");
    const int B = cfgs[0].num_bitplanes;
    for (int f = 0; f < nfields; f++) {
        const prodm_config& c = cfgs[f];
        if (c.dtype != PRODM_F32 || c.encoder != PRODM_ENC_NEGABINARY || c.basis != PRODM_BASIS_HIERARCHICAL)
            return fail(PRODM_EUNSUPPORTED, "batched fields: fp32, negabinary, hierarchical basis");
        if (c.num_bitplanes != B || B < 1 || B > 32) return fail(PRODM_EINVAL, "batched fields share 1..32 bitplanes");
        if (c.ndims < 1 || c.ndims > 3) return fail(PRODM_EINVAL, "ndims must be 1, 2 or 3");
        int ml = max_level(c.ndims, c.dims);
        if (c.target_level < 0 || c.target_level > ml)
            return fail(PRODM_EINVAL, "field " + std::to_string(f) + ": target level is higher than " + std::to_string(ml));
    }
    prodm_batch* h = new prodm_batch();
    h->nf = nfields;
    h->B = B;
    h->cfg.assign(cfgs, cfgs + nfields);
    h->g.resize(nfields);
    uint64_t coef = 0, rcoef = 0, cb = 0, sb = 0;
    h->coef_off.resize(nfields);
    h->rcoef_off.resize(nfields);
    h->roff.resize(nfields);
    h->cb_off.resize(nfields);
    h->cb_len.resize(nfields);
    h->lvl_stream_off.resize(nfields);
    int rc;
    std::vector<int> levels(nfields), ndims(nfields);
    for (int f = 0; f < nfields; f++) {
        if ((rc = make_geom(cfgs[f].ndims, cfgs[f].dims, cfgs[f].target_level, h->g[f]))) { delete h; return rc; }
        const LevelGeom& g = h->g[f];
        h->maxL = std::max(h->maxL, g.L);
        levels[f] = g.L;
        ndims[f] = g.ndims;
        h->coef_off[f] = coef;
        coef += (g.total + 63) & ~(uint64_t)63;
        h->roff[f].assign(g.L + 2, 0);
        for (int l = 0; l <= g.L; l++) h->roff[f][l + 1] = (h->roff[f][l] + g.elems[l] + 3) / 4 * 4;
        h->rcoef_off[f] = rcoef;
        rcoef += (h->roff[f][g.L + 1] + 63) & ~(uint64_t)63;
        h->cb_off[f] = cb;
        h->cb_len[f] = g.L >= 1 ? ((g.box[g.L - 1].size() + 63) & ~(uint64_t)63) : 64;
        cb += 2 * h->cb_len[f];
        h->lvl_stream_off[f].resize(g.L + 1);
        for (int l = 0; l <= g.L; l++) {
            h->lvl_stream_off[f][l] = sb;
            sb += (uint64_t)B * (((g.elems[l] + 31) / 32 + 3) / 4 * 4) * 4;
            sb = (sb + 255) & ~(uint64_t)255;
        }
    }
    const size_t slots = (size_t)nfields * kMaxL;
    if ((rc = h->alloc((void**)&h->coef, coef * 4)) || (rc = h->alloc((void**)&h->rcoef, rcoef * 4)) ||
        (rc = h->alloc((void**)&h->cbuf, cb * 4)) || (rc = h->alloc((void**)&h->rbuf, cb * 4)) ||
        (rc = h->alloc((void**)&h->streams, sb)) || (rc = h->alloc((void**)&h->keys, slots * 4)) ||
        (rc = h->alloc((void**)&h->bounds, slots * 4)) || (rc = h->alloc((void**)&h->sizes, slots * B * 4)) ||
        (rc = h->alloc((void**)&h->maxerr, slots * (B + 1) * 8)) || (rc = h->alloc((void**)&h->index, slots)) ||
        (rc = h->alloc((void**)&h->rsz, slots * 4)) || (rc = h->alloc((void**)&h->ndims_d, nfields * 4)) ||
        (rc = h->alloc((void**)&h->levels_d, nfields * 4)) || (rc = h->alloc((void**)&h->tols, nfields * 8)) ||
        (rc = h->alloc((void**)&h->kstatus, 16))) {
        delete h;
        return rc;
    }
    std::vector<uint32_t> sz(slots * B, 0);
    for (int f = 0; f < nfields; f++)
        for (int l = 0; l <= h->g[f].L; l++)
            for (int p = 0; p < B; p++) sz[((size_t)f * kMaxL + l) * B + p] = (uint32_t)(((h->g[f].elems[l] + 31) / 32) * 4);
    cudaError_t e = cudaMemcpy(h->sizes, sz.data(), sz.size() * 4, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(h->levels_d, levels.data(), nfields * 4, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(h->ndims_d, ndims.data(), nfields * 4, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemset(h->index, 0, slots);
    if (e == cudaSuccess) e = cudaMemset(h->maxerr, 0, slots * (B + 1) * 8);
    if (e == cudaSuccess) e = cudaMemset(h->kstatus, 0, 16);
    if (e != cudaSuccess) { delete h; return cuda_status(e, "prodm_batch_create"); }
    *out = h;
    return PRODM_OK;
}

int prodm_batch_bind(prodm_batch* h, const void* const* d_fields, void* const* d_outs) {
    if (!h || !d_fields || !d_outs) return fail(PRODM_EINVAL, "prodm_batch_bind: NULL pointer");
    h->fields.assign((const float* const*)d_fields, (const float* const*)d_fields + h->nf);
    h->outs.assign((float* const*)d_outs, (float* const*)d_outs + h->nf);
    h->bound = true;
    return batch_build_segments(h);
}

int prodm_batch_set_stage_launch(prodm_batch* h, int stage, int threads_per_cta, int ctas_per_sm) {
    if (!h) return fail(PRODM_EINVAL, "NULL handle");
    if (stage < PRODM_BATCH_DECOMPOSE || stage > PRODM_BATCH_FUSED) return fail(PRODM_EINVAL, "unknown batch stage");
    if (stage == PRODM_BATCH_ENCODE || stage == PRODM_BATCH_FUSED) {
        if (threads_per_cta != 256) return fail(PRODM_EINVAL, "the encode and fused stages run 256 threads per CTA");
        if (ctas_per_sm < 1 || ctas_per_sm > 8) return fail(PRODM_EINVAL, "encode / fused CTAs per SM must be in [1, 8]");
    } else {
        if (threads_per_cta != 64 && threads_per_cta != 128 && threads_per_cta != 256)
            return fail(PRODM_EINVAL, "threads per CTA must be 64, 128 or 256");
        if (ctas_per_sm < 1 || ctas_per_sm > 32) return fail(PRODM_EINVAL, "CTAs per SM must be in [1, 32]");
    }
    h->st_threads[stage] = threads_per_cta;
    h->st_ctas[stage] = ctas_per_sm;
    return PRODM_OK;
}

int prodm_batch_set_fused_unit(prodm_batch* h, int values_per_unit) {
    if (!h) return fail(PRODM_EINVAL, "NULL handle");
    if (values_per_unit < 256 || values_per_unit > 8192)
        return fail(PRODM_EINVAL, "values per fused unit must be in [256, 8192]");
    h->unit_values = (uint32_t)values_per_unit;
    return h->bound ? batch_build_segments(h) : PRODM_OK;
}

int prodm_batch_set_launch(prodm_batch* h, int threads_per_cta, int ctas_per_sm) {
    if (!h) return fail(PRODM_EINVAL, "NULL handle");
    if (threads_per_cta != 64 && threads_per_cta != 128 && threads_per_cta != 256)
        return fail(PRODM_EINVAL, "threads per CTA must be 64, 128 or 256");
    if (ctas_per_sm < 1 || ctas_per_sm > 32) return fail(PRODM_EINVAL, "CTAs per SM must be in [1, 32]");
    for (int st = PRODM_BATCH_DECOMPOSE; st <= PRODM_BATCH_RECOMPOSE; st += 2) {
        h->st_threads[st] = threads_per_cta;
        h->st_ctas[st] = ctas_per_sm;
    }
    h->st_ctas[PRODM_BATCH_ENCODE] = ctas_per_sm < 8 ? ctas_per_sm : 8;
    return PRODM_OK;
}

int prodm_batch_refactor(prodm_batch* h, void* stream) {
    if (!h || !h->bound) return fail(PRODM_EINVAL, "prodm_batch_refactor: bind the field buffers first");
    return batch_refactor(h, (cudaStream_t)stream);
}

int prodm_batch_set_tolerances(prodm_batch* h, const double* h_tols, void* stream) {
    if (!h || !h_tols) return fail(PRODM_EINVAL, "NULL pointer");
    PRODM_CUDA(cudaMemcpyAsync(h->tols, h_tols, h->nf * 8, cudaMemcpyHostToDevice, (cudaStream_t)stream));
    PRODM_CUDA(cudaStreamSynchronize((cudaStream_t)stream));
    return PRODM_OK;
}

int prodm_batch_retrieve(prodm_batch* h, int interpreter, int estimator, double s, void* stream) {
    if (!h || !h->bound) return fail(PRODM_EINVAL, "prodm_batch_retrieve: bind the field buffers first");
    if (estimator != PRODM_EST_MAX_HB && estimator != PRODM_EST_MAX_OB)
        return fail(PRODM_EUNSUPPORTED, "batched retrieval uses the max-error estimators");
    if (interpreter < 0 || interpreter > 2) return fail(PRODM_EINVAL, "unknown interpreter");
    return batch_retrieve(h, interpreter, estimator, s, (cudaStream_t)stream);
}

int prodm_batch_reset(prodm_batch* h, void* stream) {
    if (!h) return fail(PRODM_EINVAL, "NULL handle");
    PRODM_CUDA(cudaMemsetAsync(h->index, 0, (size_t)h->nf * kMaxL, (cudaStream_t)stream));
    return PRODM_OK;
}

int prodm_batch_field_info(prodm_batch* h, int field, uint8_t* h_index, uint32_t* h_sizes, double* h_bounds,
                           void* stream) {
    if (!h || field < 0 || field >= h->nf) return fail(PRODM_EINVAL, "bad field");
    cudaStream_t st = (cudaStream_t)stream;
    const int nl = h->g[field].L + 1, B = h->B;
    if (h_index) PRODM_CUDA(cudaMemcpyAsync(h_index, h->index + field * kMaxL, nl, cudaMemcpyDeviceToHost, st));
    if (h_sizes) PRODM_CUDA(cudaMemcpyAsync(h_sizes, h->sizes + (size_t)field * kMaxL * B, (size_t)nl * B * 4, cudaMemcpyDeviceToHost, st));
    std::vector<float> b(nl);
    if (h_bounds) PRODM_CUDA(cudaMemcpyAsync(b.data(), h->bounds + field * kMaxL, nl * 4, cudaMemcpyDeviceToHost, st));
    PRODM_CUDA(cudaStreamSynchronize(st));
    if (h_bounds) for (int l = 0; l < nl; l++) h_bounds[l] = b[l];
    return PRODM_OK;
}

int prodm_batch_export_level(prodm_batch* h, int field, int level, void* dst, uint64_t cap, int dst_is_host,
                             uint64_t* len, void* stream) {
    if (!h || field < 0 || field >= h->nf || level < 0 || level > h->g[field].L) return fail(PRODM_EINVAL, "bad field/level");
    const uint64_t bytes = (uint64_t)h->B * ((h->g[field].elems[level] + 31) / 32) * 4;
    if (len) *len = bytes;
    if (!dst) return PRODM_OK;
    if (cap < bytes) return fail(PRODM_EINVAL, "export buffer too small");
    cudaStream_t st = (cudaStream_t)stream;
    const uint64_t nbk = (h->g[field].elems[level] + 31) / 32;
    PRODM_CUDA(cudaMemcpy2DAsync(dst, nbk * 4, h->streams + h->lvl_stream_off[field][level], (nbk + 3) / 4 * 16, nbk * 4,
                                 h->B, dst_is_host ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice, st));
    PRODM_CUDA(cudaStreamSynchronize(st));
    return PRODM_OK;
}

int prodm_batch_status(prodm_batch* h, void* stream) {
    if (!h) return fail(PRODM_EINVAL, "NULL handle");
    cudaStream_t st = (cudaStream_t)stream;
    int code = 0;
    PRODM_CUDA(cudaMemcpyAsync(&code, h->kstatus, 4, cudaMemcpyDeviceToHost, st));
    PRODM_CUDA(cudaMemsetAsync(h->kstatus, 0, 4, st));
    PRODM_CUDA(cudaStreamSynchronize(st));
    if (code == PRODM_ETIMEOUT) return fail(code, "a batched fused kernel's wait for its plane tiles ran out");
    if (code) return fail(code, "a batched fused kernel reported an error");
    return PRODM_OK;
}

int prodm_batch_destroy(prodm_batch* h) {
    delete h;
    return PRODM_OK;
}

}  // extern "C"
