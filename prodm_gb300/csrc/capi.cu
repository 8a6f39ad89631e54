// C ABI of the GB300 MDR path: component entry points (the reference's plugin
// concepts) and the device-resident composed refactor / reconstructor.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "common.cuh"
#include "kernels.cuh"

namespace prodm {

namespace {
thread_local std::string g_err;
std::atomic<uint64_t> g_launches{0};
}
void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }
bool pdl_enabled() {
    static const bool on = [] {
        const char* v = getenv("PRODM_NO_PDL");
        return !(v && v[0] == '1');
    }();
    return on;
}
void set_error(const std::string& msg) { g_err = msg; }
bool zstd_available();
int zstd_expand_plane(const uint8_t* src, uint64_t stored, uint64_t max_raw, std::vector<uint8_t>& out);

int fail(int status, const std::string& msg) {
    g_err = msg;
    return status;
}
int cuda_status(cudaError_t e, const char* where) {
    g_err = std::string(where) + ": " + cudaGetErrorString(e);
    return e == cudaErrorMemoryAllocation ? PRODM_ENOMEM : PRODM_ECUDA;
}

int device_sms() {
    static std::mutex mu;
    static std::vector<std::pair<int, int>> cache;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) dev = 0;
    std::lock_guard<std::mutex> lock(mu);
    for (const auto& e : cache)
        if (e.first == dev) return e.second;
    int sms = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms < 1) sms = kSMs;
    (void)cudaGetLastError();
    cache.push_back({dev, sms});
    return sms;
}

unsigned resident_ctas(const void* kernel, int threads, size_t smem) {
    struct Entry {
        int dev;
        const void* k;
        int threads;
        size_t smem;
        unsigned ctas;
    };
    static std::mutex mu;
    static std::vector<Entry> cache;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) dev = 0;
    {
        std::lock_guard<std::mutex> lock(mu);
        for (const Entry& e : cache)
            if (e.dev == dev && e.k == kernel && e.threads == threads && e.smem == smem) return e.ctas;
    }
    const int sms = device_sms();
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, smem) != cudaSuccess || per_sm < 1)
        per_sm = 1;
    (void)cudaGetLastError();
    const unsigned ctas = (unsigned)(sms * per_sm);
    std::lock_guard<std::mutex> lock(mu);
    cache.push_back({dev, kernel, threads, smem, ctas});
    return ctas;
}

int max_level(int ndims, const uint32_t* dims) {
    uint32_t m = dims[0];
    for (int i = 1; i < ndims; i++) m = dims[i] < m ? dims[i] : m;
    return (int)(uint8_t)(std::log2((double)m) - 1);   // ComposedRefactor.hpp:79
}

int make_geom(int ndims, const uint32_t* dims, int L, LevelGeom& g) {
    if (ndims < 1 || ndims > 3) return fail(PRODM_EINVAL, "ndims must be 1, 2 or 3");
    if (L < 0 || L > 16) return fail(PRODM_EINVAL, "target level must be in [0, 16]");
    for (int i = 0; i < ndims; i++)
        if (dims[i] == 0) return fail(PRODM_EINVAL, "zero-sized dimension");
    g.ndims = ndims;
    g.L = L;
    for (int i = 0; i < 3; i++) g.dims[i] = i < ndims ? dims[i] : 0;
    Box top;
    for (int i = 0; i < 3; i++) top.n[i] = i < 3 - ndims ? 1 : dims[i - (3 - ndims)];
    g.box[L] = top;
    for (int l = L; l >= 1; l--)
        for (int i = 0; i < 3; i++) g.box[l - 1].n[i] = coarse_len(g.box[l].n[i]);
    uint64_t off = 0, prev = 0;
    for (int l = 0; l <= L; l++) {
        uint64_t v = g.box[l].size();
        g.elems[l] = v - prev;
        g.offset[l] = off;
        off += g.elems[l];
        prev = v;
    }
    g.total = off;
    return PRODM_OK;
}

// stream-ordered scratch: caller-provided memory or cudaMallocAsync
class Workspace {
  public:
    Workspace(void* base, size_t bytes, cudaStream_t st) : base_((uint8_t*)base), cap_(bytes), st_(st) {}
    ~Workspace() {
        if (owned_) cudaFreeAsync(base_, st_);
    }
    static size_t align(size_t x) { return (x + 255) & ~(size_t)255; }
    void reserve(size_t b) { need_ += align(b); }
    int commit() {
        if (base_) {
            if (cap_ < need_) return fail(PRODM_EINVAL, "workspace too small: need " + std::to_string(need_) + " bytes");
            return PRODM_OK;
        }
        if (need_ == 0) return PRODM_OK;
        cudaError_t e = cudaMallocAsync((void**)&base_, need_, st_);
        if (e != cudaSuccess) return cuda_status(e, "cudaMallocAsync(workspace)");
        owned_ = true;
        cap_ = need_;
        return PRODM_OK;
    }
    void* take(size_t b) {
        void* p = base_ + used_;
        used_ += align(b);
        return p;
    }
    size_t needed() const { return need_; }

  private:
    uint8_t* base_;
    size_t cap_;
    size_t need_ = 0, used_ = 0;
    cudaStream_t st_;
    bool owned_ = false;
};

size_t esize(int dtype) { return dtype == PRODM_F64 ? 8 : 4; }
int block_of(int dtype) { return dtype == PRODM_F64 ? 64 : 32; }

int check_dtype(int dtype) {
    if (dtype != PRODM_F32 && dtype != PRODM_F64) return fail(PRODM_EINVAL, "dtype must be PRODM_F32 or PRODM_F64");
    return PRODM_OK;
}
int check_bitplanes(int dtype, int enc, int B) {
    int maxB = dtype == PRODM_F64 ? (enc == PRODM_ENC_NEGABINARY ? 64 : 63) : 32;
    if (B < 1 || B > maxB) return fail(PRODM_EINVAL, "num_bitplanes must be in [1, " + std::to_string(maxB) + "]");
    return PRODM_OK;
}

// strides (elements) of dims 0 and 1 of the padded 3-D view
int view_strides(int ndims, const uint32_t* dims, const uint32_t* strides, uint64_t& s0, uint64_t& s1) {
    uint64_t d[3];
    for (int i = 0; i < 3; i++) d[i] = i < 3 - ndims ? 1 : dims[i - (3 - ndims)];
    if (!strides) {
        s0 = d[1] * d[2];
        s1 = d[2];
        return PRODM_OK;
    }
    if (strides[ndims - 1] != 1) return fail(PRODM_EUNSUPPORTED, "the innermost stride must be 1");
    if (ndims == 3) { s0 = strides[0]; s1 = strides[1]; }
    else if (ndims == 2) { s0 = 0; s1 = strides[0]; }
    else { s0 = 0; s1 = 0; }
    return PRODM_OK;
}

// ---------------------------------------------------------------------------
// decomposer
// ---------------------------------------------------------------------------
struct OrthScratch {
    void* fnat = nullptr;
    void* t1 = nullptr;
    void* t2 = nullptr;
    void* z = nullptr;
};

void orth_reserve(Workspace& ws, const Box& F, size_t es) {
    Box C{{coarse_len(F.n[0]), coarse_len(F.n[1]), coarse_len(F.n[2])}};
    ws.reserve(F.size() * es);
    ws.reserve((uint64_t)F.n[0] * F.n[1] * C.n[2] * es);
    ws.reserve((uint64_t)F.n[0] * C.n[1] * C.n[2] * es);
    ws.reserve(C.size() * es);
}
OrthScratch orth_take(Workspace& ws, const Box& F, size_t es) {
    Box C{{coarse_len(F.n[0]), coarse_len(F.n[1]), coarse_len(F.n[2])}};
    OrthScratch o;
    o.fnat = ws.take(F.size() * es);
    o.t1 = ws.take((uint64_t)F.n[0] * F.n[1] * C.n[2] * es);
    o.t2 = ws.take((uint64_t)F.n[0] * C.n[1] * C.n[2] * es);
    o.z = ws.take(C.size() * es);
    return o;
}
size_t tab_elems(const LevelGeom& g) {
    size_t t = 0;
    for (int l = 1; l <= g.L; l++)
        for (int d = 0; d < 3; d++) t += 3 * (size_t)coarse_len(g.box[l].n[d]);
    return t;
}
// host tables for all levels; offsets[l*3+d] in elements
template <class T>
std::vector<T> build_tabs(const LevelGeom& g, std::vector<size_t>& offsets) {
    std::vector<T> tab(tab_elems(g) + 1);
    offsets.assign(3 * (g.L + 1), 0);
    size_t o = 0;
    for (int l = 1; l <= g.L; l++)
        for (int d = 0; d < 3; d++) {
            offsets[l * 3 + d] = o;
            mass_factors<T>(g.box[l].n[d], tab.data() + o);
            o += 3 * (size_t)coarse_len(g.box[l].n[d]);
        }
    return tab;
}

template <class T>
int decompose_impl(T* data, int ndims, const uint32_t* dims, int L, const uint32_t* strides, int basis, void* wsp,
                   size_t wsb, cudaStream_t st, bool inverse) {
    LevelGeom g;
    int rc = make_geom(ndims, dims, L, g);
    if (rc) return rc;
    uint64_t s0, s1;
    if ((rc = view_strides(ndims, dims, strides, s0, s1))) return rc;
    if (L == 0) return PRODM_OK;
    const bool orth = basis == PRODM_BASIS_ORTHOGONAL;
    const Box& top = g.box[L];
    Workspace ws(wsp, wsb, st);
    ws.reserve(top.size() * sizeof(T));
    if (orth) {
        orth_reserve(ws, top, sizeof(T));
        ws.reserve((tab_elems(g) + 1) * sizeof(T));
    }
    if ((rc = ws.commit())) return rc;
    T* scratch = (T*)ws.take(top.size() * sizeof(T));
    OrthScratch os;
    T* dtab = nullptr;
    std::vector<size_t> toff;
    if (orth) {
        os = orth_take(ws, top, sizeof(T));
        std::vector<T> tab = build_tabs<T>(g, toff);
        dtab = (T*)ws.take(tab.size() * sizeof(T));
        PRODM_CUDA(cudaMemcpyAsync(dtab, tab.data(), tab.size() * sizeof(T), cudaMemcpyHostToDevice, st));
        PRODM_CUDA(cudaStreamSynchronize(st));   // host table lifetime
    }
    for (int step = 0; step < L; step++) {
        const int l = inverse ? step + 1 : L - step;
        const Box& F = g.box[l];
        const Box& C = g.box[l - 1];
        const uint64_t f0 = (uint64_t)F.n[1] * F.n[2], f1 = F.n[2];
        if ((rc = launch_copy_box<T>(data, s0, s1, F, scratch, f0, f1, st))) return rc;
        const T* tabs[3] = {nullptr, nullptr, nullptr};
        if (orth)
            for (int d = 0; d < 3; d++) tabs[d] = dtab + toff[l * 3 + d];
        if (!inverse) {
            if ((rc = launch_decompose_level_inplace<T>(scratch, F, C, data, s0, s1, orth ? (T*)os.fnat : nullptr, st)))
                return rc;
            if (orth) {
                if ((rc = launch_l2_correction<T>((T*)os.fnat, F, (T*)os.t1, (T*)os.t2, (T*)os.z, tabs, st))) return rc;
                if ((rc = launch_add_box<T>(data, s0, s1, (T*)os.z, C, (T)1, st))) return rc;
            }
        } else {
            if (orth) {
                if ((rc = launch_reordered_to_natural<T>(scratch, F, C, (T*)os.fnat, st))) return rc;
                if ((rc = launch_l2_correction<T>((T*)os.fnat, F, (T*)os.t1, (T*)os.t2, (T*)os.z, tabs, st))) return rc;
                if ((rc = launch_add_box<T>(scratch, f0, f1, (T*)os.z, C, (T)-1, st))) return rc;
            }
            if ((rc = launch_recompose_level_inplace<T>(scratch, F, C, data, s0, s1, st))) return rc;
        }
    }
    return PRODM_OK;
}

int decompose_ws_bytes(int dtype, int ndims, const uint32_t* dims, int L, int basis, size_t* bytes) {
    LevelGeom g;
    int rc = make_geom(ndims, dims, L, g);
    if (rc) return rc;
    size_t es = esize(dtype);
    Workspace ws(nullptr, 0, 0);
    ws.reserve(g.box[L].size() * es);
    if (basis == PRODM_BASIS_ORTHOGONAL) {
        orth_reserve(ws, g.box[L], es);
        ws.reserve((tab_elems(g) + 1) * es);
    }
    *bytes = ws.needed();
    return PRODM_OK;
}

// ---------------------------------------------------------------------------
// encoder
// ---------------------------------------------------------------------------
uint64_t nblocks_of(int dtype, uint64_t n) { return (n + block_of(dtype) - 1) / block_of(dtype); }

uint64_t encode_bound(int enc, int dtype, uint64_t n, int B) {
    uint64_t nb = nblocks_of(dtype, n);
    uint64_t wb = esize(dtype);
    if (enc == PRODM_ENC_NEGABINARY) return (uint64_t)B * nb * wb;
    if (enc == PRODM_ENC_PERBIT) return (uint64_t)B * ((2 * n + 63) / 64 * 8);   // <= 2 bits per value and plane
    return (uint64_t)B * nb * wb + nb * wb + 4 + nb;   // each block: rb header + (B - rb) words + one sign word
}

void encode_reserve(Workspace& ws, int enc, int dtype, uint64_t n, int B) {
    uint64_t nb = nblocks_of(dtype, n);
    uint64_t nch = gr_nchunks(nb);
    uint64_t parts = nch > (uint64_t)kPartialSlots ? nch : (uint64_t)kPartialSlots;
    ws.reserve(partial_bytes(parts, B));
    if (enc == PRODM_ENC_PERBIT) {
        ws.reserve((uint64_t)(B + 1) * pb_row_words(n) * 4);   // magnitude + sign rows
        ws.reserve(64 * 4);                                    // first-one counts
        ws.reserve(pb_pack_scratch_bytes(n, B));
    }
    if (enc == PRODM_ENC_GROUPED) {
        ws.reserve((uint64_t)B * 2 * nb * esize(dtype));  // aligned staging
        ws.reserve(nb);                                   // rb
        ws.reserve(nch * B * 4);                          // chunk words
        ws.reserve(nch * B * 4);                          // chunk offsets
        ws.reserve(64 * sizeof(void*));                   // plane pointers
    }
}

template <class T>
int encode_impl(int enc, const T* x, uint64_t n, int exp, int B, uint8_t* blob, uint64_t cap, uint32_t* sizes,
                double* errs, void* wsp, size_t wsb, cudaStream_t st) {
    const int dtype = sizeof(T) == 8 ? PRODM_F64 : PRODM_F32;
    int rc;
    if (n == 0) return fail(PRODM_EINVAL, "encode: n must be >= 1");
    if ((rc = check_bitplanes(dtype, enc, B))) return rc;
    if (cap < encode_bound(enc, dtype, n, B)) return fail(PRODM_EINVAL, "encode: blob capacity below prodm_encode_bound");
    const uint64_t nb = nblocks_of(dtype, n);
    const uint64_t nch = gr_nchunks(nb);
    const uint64_t parts = nch > (uint64_t)kPartialSlots ? nch : (uint64_t)kPartialSlots;
    Workspace ws(wsp, wsb, st);
    encode_reserve(ws, enc, dtype, n, B);
    if ((rc = ws.commit())) return rc;
    double* partial = (double*)ws.take(partial_bytes(parts, B));
    if (enc == PRODM_ENC_PERBIT) {
        if ((uintptr_t)blob % 8) return fail(PRODM_EINVAL, "encode: the per-bit blob must be 8-byte aligned");
        const uint64_t rw = pb_row_words(n);
        uint32_t* rows = (uint32_t*)ws.take((uint64_t)(B + 1) * rw * 4);
        uint32_t* counts = (uint32_t*)ws.take(64 * 4);
        void* scratch = ws.take(pb_pack_scratch_bytes(n, B));
        if ((rc = launch_pb_encode<T>(x, n, nullptr, exp, B, rows, rw, counts, sizes, st))) return rc;
        return launch_pb_pack(rows, rw, n, B, sizes, encode_bound(enc, dtype, n, B), blob, scratch, st);
    }
    if (enc == PRODM_ENC_NEGABINARY) {
        if ((uintptr_t)blob % sizeof(T)) return fail(PRODM_EINVAL, "encode: blob must be aligned to the stream word");
        if ((rc = launch_fill_u32(sizes, (uint64_t)B, (uint32_t)(nb * sizeof(T)), st))) return rc;
        return launch_nb_encode<T>(x, n, nullptr, exp, B, blob, nb, partial, errs, st);
    }
    uint8_t* staging = (uint8_t*)ws.take((uint64_t)B * 2 * nb * sizeof(T));
    uint8_t* rbs = (uint8_t*)ws.take(nb);
    uint32_t* cw = (uint32_t*)ws.take(nch * B * 4);
    uint32_t* co = (uint32_t*)ws.take(nch * B * 4);
    void** dptrs = (void**)ws.take(64 * sizeof(void*));
    if ((rc = launch_gr_encode<T>(x, n, nullptr, exp, B, rbs, cw, co, sizes, staging, 2 * nb, partial, errs, st)))
        return rc;
    std::vector<void*> ptrs(B);
    for (int p = 0; p < B; p++) ptrs[p] = staging + (uint64_t)p * 2 * nb * sizeof(T);
    PRODM_CUDA(cudaMemcpyAsync(dptrs, ptrs.data(), B * sizeof(void*), cudaMemcpyHostToDevice, st));
    PRODM_CUDA(cudaStreamSynchronize(st));
    return launch_gr_pack(dptrs, sizes, B, nb, rbs, (int)sizeof(T), blob, st);
}

}  // namespace prodm

using namespace prodm;

// ---------------------------------------------------------------------------
// stateful progressive decoder
// ---------------------------------------------------------------------------
struct prodm_decoder {
    int enc;
    int dtype;
    struct Level {
        bool have = false;
        uint64_t n = 0;
        int B = 0;
        uint8_t* rbs = nullptr;
        uint32_t* chunk_off = nullptr;
        void* signs = nullptr;
        uint32_t* pbrows = nullptr;   // per-bit: rows 0..B-1, sign row, unseen row, status word
        int parsed = 0;               // per-bit: planes decoded so far
    };
    std::vector<Level> levels;
    ~prodm_decoder() {
        for (auto& l : levels) {
            if (l.pbrows) cudaFree(l.pbrows);
            if (l.rbs) cudaFree(l.rbs);
            if (l.chunk_off) cudaFree(l.chunk_off);
            if (l.signs) cudaFree(l.signs);
        }
    }
};

namespace prodm {
namespace {
// per-bit levels: parse planes [s, s+num) of the reference streams into the
// level's rows (the unseen / sign rows carry the state of the planes before),
// then decode their contribution
template <class T>
int pb_progressive_decode(prodm_decoder* h, const uint8_t* blob, const uint32_t* hs, uint64_t n, int exp, int s,
                          int num, int level, int B, T* out, cudaStream_t st) {
    if (B > (sizeof(T) == 8 ? 63 : 32)) return fail(PRODM_EINVAL, "decode: per-bit fp64 streams hold at most 63 planes");
    if ((int)h->levels.size() <= level) h->levels.resize(level + 1);
    auto& L = h->levels[level];
    const uint64_t rw = pb_row_words(n);
    if (!L.have) {
        if (s != 0) return fail(PRODM_EINVAL, "decode: the first call for a level must start at plane 0");
        if (L.pbrows && (L.n != n || L.B != B)) { cudaFree(L.pbrows); L.pbrows = nullptr; }
        if (!L.pbrows) PRODM_CUDA(cudaMalloc((void**)&L.pbrows, (uint64_t)(B + 2) * rw * 4 + 16));
        int rc = launch_pb_init_unseen(L.pbrows + (uint64_t)(B + 1) * rw, L.pbrows + (uint64_t)B * rw, n, st);
        if (rc) return rc;
        L.have = true;
        L.n = n;
        L.B = B;
        L.parsed = 0;
    } else if (L.n != n || L.B != B) {
        return fail(PRODM_EINVAL, "decode: level shape changed between calls");
    }
    if (s != L.parsed)
        return fail(PRODM_EINVAL, "decode: per-bit planes are decoded in order; this level continues at plane " +
                                      std::to_string(L.parsed));
    uint64_t total = 0;
    for (int i = 0; i < num; i++) {
        if (hs[i] % 8 || hs[i] == 0) return fail(PRODM_ECORRUPT, "decode: per-bit stream size not a positive multiple of 8");
        total += hs[i];
    }
    uint32_t* rows = L.pbrows;
    int* status = (int*)(rows + (uint64_t)(B + 2) * rw);
    uint8_t* tmp = nullptr;
    const uint8_t* base = blob;
    if ((uintptr_t)blob % 8) {   // streams are read as 64-bit words
        PRODM_CUDA(cudaMallocAsync((void**)&tmp, total, st));
        PRODM_CUDA(cudaMemcpyAsync(tmp, blob, total, cudaMemcpyDeviceToDevice, st));
        base = tmp;
    }
    std::vector<uint64_t> hv(2 * num);
    uint64_t o = 0;
    for (int i = 0; i < num; i++) {
        hv[i] = (uint64_t)(uintptr_t)(base + o);
        hv[num + i] = hs[i] / 8;
        o += hs[i];
    }
    uint64_t* dv;   // plane pointers, word counts, then the parse pipeline's scratch
    const size_t head = (hv.size() * 8 + 255) / 256 * 256;
    PRODM_CUDA(cudaMallocAsync((void**)&dv, head + pb_parse_scratch_bytes(num), st));
    PRODM_CUDA(cudaMemcpyAsync(dv, hv.data(), hv.size() * 8, cudaMemcpyHostToDevice, st));
    PRODM_CUDA(cudaMemsetAsync(status, 0, 4, st));
    int rc = launch_pb_parse((const uint64_t* const*)dv, dv + num, s, num, n, rows, rw, rows + (uint64_t)(B + 1) * rw,
                             rows + (uint64_t)B * rw, (uint8_t*)dv + head, status, st);
    if (!rc)
        rc = launch_pb_decode<T>(rows, rw, n, nullptr, exp, B, s, s + num, nullptr, rows + (uint64_t)B * rw,
                                 rows + (uint64_t)(B + 1) * rw, out, st);
    int hstat = 0;
    if (!rc) {
        cudaError_t e = cudaMemcpyAsync(&hstat, status, 4, cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) rc = cuda_status(e, "per-bit decode");
    }
    cudaFreeAsync(dv, st);
    if (tmp) cudaFreeAsync(tmp, st);
    // a failed parse leaves the level's state behind the data: the next call
    // for this level starts again at plane 0
    if (rc || hstat) L.have = false;
    if (rc) return rc;
    if (hstat == PRODM_ETIMEOUT) return fail(PRODM_ETIMEOUT, "decode: the per-bit parse pipeline stalled");
    if (hstat) return fail(PRODM_ECORRUPT, "decode: a per-bit stream does not end where its size says");
    L.parsed = s + num;
    return PRODM_OK;
}

template <class T>
int progressive_decode_impl(prodm_decoder* h, const uint8_t* blob, const uint32_t* hs, uint64_t n, int exp, int s,
                            int num, int level, int B, T* out, cudaStream_t st) {
    const int dtype = sizeof(T) == 8 ? PRODM_F64 : PRODM_F32;
    const int ws_ = (int)sizeof(T);
    if (num == 0) {
        PRODM_CUDA(cudaMemsetAsync(out, 0, n * sizeof(T), st));
        return PRODM_OK;
    }
    if (n == 0) return fail(PRODM_EINVAL, "decode: n must be >= 1");
    if (s < 0 || num < 0 || s + num > B) return fail(PRODM_EINVAL, "decode: planes outside [0, total_bitplanes)");
    if (h->enc == PRODM_ENC_PERBIT) return pb_progressive_decode<T>(h, blob, hs, n, exp, s, num, level, B, out, st);
    const uint64_t nb = nblocks_of(dtype, n);
    int rc;
    if (h->enc == PRODM_ENC_NEGABINARY) {
        for (int i = 0; i < num; i++)
            if (hs[i] != nb * sizeof(T)) return fail(PRODM_ECORRUPT, "decode: negabinary stream size mismatch");
        if ((uintptr_t)blob % sizeof(T) == 0)
            return launch_nb_decode<T>(blob, nb, n, nullptr, exp, s, num, nullptr, out, st);
        // misaligned planes: copy to aligned scratch first
        void* tmp;
        PRODM_CUDA(cudaMallocAsync(&tmp, (uint64_t)num * nb * sizeof(T), st));
        PRODM_CUDA(cudaMemcpyAsync(tmp, blob, (uint64_t)num * nb * sizeof(T), cudaMemcpyDeviceToDevice, st));
        rc = launch_nb_decode<T>(tmp, nb, n, nullptr, exp, s, num, nullptr, out, st);
        cudaFreeAsync(tmp, st);
        return rc;
    }
    if ((int)h->levels.size() <= level) h->levels.resize(level + 1);
    auto& L = h->levels[level];
    const uint64_t nch = gr_nchunks(nb);
    uint64_t hdr = 0;
    if (!L.have) {
        if (s != 0) return fail(PRODM_EINVAL, "decode: the first call for a level must start at plane 0");
        if (hs[0] < 4 + nb) return fail(PRODM_ECORRUPT, "decode: stream 0 shorter than its header");
        uint32_t cnt = 0;
        PRODM_CUDA(cudaMemcpyAsync(&cnt, blob, 4, cudaMemcpyDeviceToHost, st));
        PRODM_CUDA(cudaStreamSynchronize(st));
        if (cnt != nb) return fail(PRODM_ECORRUPT, "decode: block count in stream 0 does not match n");
        PRODM_CUDA(cudaMalloc(&L.rbs, nb));
        PRODM_CUDA(cudaMalloc(&L.chunk_off, nch * B * 4));
        PRODM_CUDA(cudaMalloc(&L.signs, nb * sizeof(T)));
        PRODM_CUDA(cudaMemcpyAsync(L.rbs, blob + 4, nb, cudaMemcpyDeviceToDevice, st));
        uint32_t* cw;
        uint32_t* sz;
        PRODM_CUDA(cudaMallocAsync((void**)&cw, nch * B * 4 + 64 * 4, st));
        sz = cw + nch * B;
        if ((rc = launch_chunk_words_from_rb(L.rbs, nb, B, cw, st))) return rc;
        if ((rc = launch_gr_scan_only(cw, nch, B, nb, ws_, L.chunk_off, sz, st))) return rc;
        cudaFreeAsync(cw, st);
        L.have = true;
        L.n = n;
        L.B = B;
        hdr = 4 + nb;
    } else if (L.n != n || L.B != B) {
        return fail(PRODM_EINVAL, "decode: level shape changed between calls");
    }
    // unpack planes [s, s+num) into aligned scratch
    std::vector<uint64_t> off(num), nw(num);
    uint64_t o = 0, maxw = 0;
    for (int i = 0; i < num; i++) {
        uint64_t skip = (i == 0 && s == 0) ? hdr : 0;
        if (s == 0 && i == 0 && hdr == 0) skip = 4 + nb;
        if (hs[i] < skip || (hs[i] - skip) % sizeof(T)) return fail(PRODM_ECORRUPT, "decode: stream size not word aligned");
        off[i] = o + skip;
        nw[i] = (hs[i] - skip) / sizeof(T);
        maxw = nw[i] > maxw ? nw[i] : maxw;
        o += hs[i];
    }
    uint8_t* tmp;
    // staged planes first, then the (8-byte) offset / count / pointer arrays on a
    // 256-byte boundary
    const uint64_t plane_bytes = ((uint64_t)num * (maxw + 1) * sizeof(T) + 255) & ~(uint64_t)255;
    size_t tbytes = plane_bytes + 2 * num * 8 + B * sizeof(void*) + 256;
    PRODM_CUDA(cudaMallocAsync((void**)&tmp, tbytes, st));
    uint8_t* planes = tmp;
    uint64_t* doff = (uint64_t*)(tmp + plane_bytes);
    uint64_t* dnw = doff + num;
    void** dptr = (void**)(dnw + num);
    std::vector<void*> ptr(B, nullptr), uptr(num);
    for (int i = 0; i < num; i++) {
        uptr[i] = planes + (uint64_t)i * (maxw + 1) * sizeof(T);
        ptr[s + i] = uptr[i];
    }
    std::vector<uint8_t> hostbuf(2 * num * 8 + B * sizeof(void*));
    memcpy(hostbuf.data(), off.data(), num * 8);
    memcpy(hostbuf.data() + num * 8, nw.data(), num * 8);
    memcpy(hostbuf.data() + 2 * num * 8, ptr.data(), B * sizeof(void*));
    PRODM_CUDA(cudaMemcpyAsync(doff, hostbuf.data(), hostbuf.size(), cudaMemcpyHostToDevice, st));
    void** uptr_d;
    PRODM_CUDA(cudaMallocAsync((void**)&uptr_d, num * sizeof(void*), st));
    PRODM_CUDA(cudaMemcpyAsync(uptr_d, uptr.data(), num * sizeof(void*), cudaMemcpyHostToDevice, st));
    PRODM_CUDA(cudaStreamSynchronize(st));
    if ((rc = launch_unpack_planes(blob, doff, dnw, num, ws_, uptr_d, maxw, st))) return rc;
    rc = launch_gr_decode<T>((const void* const*)dptr, n, nullptr, exp, B, s, s + num, nullptr, L.rbs, L.chunk_off,
                             L.signs, out, st);
    cudaFreeAsync(uptr_d, st);
    cudaFreeAsync(tmp, st);
    return rc;
}
}  // namespace
}  // namespace prodm

// ---------------------------------------------------------------------------
// device-resident composed refactor / reconstructor
// ---------------------------------------------------------------------------
struct prodm_mdr {
    prodm_config cfg;
    LevelGeom g;
    int B = 0;
    size_t es = 4;
    bool nb = true, orth = false, sq = false;
    bool pb = false;                               // per-bit encoder
    // lossless stage (off while ll_latter < 0): stored sizes go to `sizes`
    // (the interpreter's cost model), the encoders' raw sizes to `rsizes`
    int ll_latter = -1;
    bool refactored = false;
    uint32_t* rsizes = nullptr;
    std::vector<uint8_t> ll_stop, ll_flags;        // per level; per level and plane
    std::vector<uint8_t*> ll_cbuf;                 // loading: stored level bytes as they arrive
    std::vector<uint64_t> ll_cloaded, ll_rawoff;   // stored bytes loaded, raw bytes expanded, per level
    std::vector<int> ll_expanded;                  // planes expanded per level
    std::vector<uint32_t> ll_stored;               // loading: stored sizes from the metadata
    // loading level files of the reference's zstd stage: their latter index
    // (AdaptiveLevelCompressor's constructor argument) and the stored bytes,
    // kept on the host until their planes are complete and expanded there
    bool ll_zstd = false;
    int zstd_latter = 26;
    std::vector<std::vector<uint8_t>> ll_hbuf;
    FileStaging* fstage = nullptr;                 // level-file reads: staging buffers
    std::vector<uint32_t> hsz;                     // host copy of `sizes` (export), valid while hsz_valid
    bool hsz_valid = false;
    uint32_t* pbcounts = nullptr;                  // per-bit: first-one counts, 64 per level
    int* pbstatus = nullptr;                       // per-bit: parse status of loaded streams
    int* kstatus = nullptr;                        // bounded device waits of retrievals (0 or a PRODM_E* code)
    uint8_t* hmap = nullptr;                       // mapped pinned host memory: plane counts [0, 64), status [64, 68)
    bool after_reconstruct = false;                // the last call on the handle was a reconstruction
    uint8_t* dmap = nullptr;                       // its device address
    std::vector<void*> allocs;
    void* coef = nullptr;
    void* cbuf[2] = {nullptr, nullptr};
    OrthScratch os;
    void* tabs = nullptr;
    std::vector<size_t> tab_off;
    uint8_t* streams = nullptr;
    std::vector<uint64_t> lvl_byte_off, plane_cap, nblocks;
    void* keys = nullptr;
    void* bounds = nullptr;
    uint32_t* sizes = nullptr;
    double* sqerr = nullptr;
    double* maxerr = nullptr;
    double* partial = nullptr;
    uint8_t* rbs = nullptr;
    std::vector<uint64_t> rb_off, co_off;
    uint32_t* chunk_words = nullptr;
    uint32_t* chunk_off = nullptr;
    void** plane_ptrs = nullptr;
    uint8_t* index = nullptr;
    uint32_t* rsz = nullptr;
    int* ndims_d = nullptr;
    int* levels_d = nullptr;
    void* rcoef = nullptr;
    std::vector<uint64_t> roff;                    // level offsets in rcoef (elements, 16-byte aligned)
    void* rbuf[2] = {nullptr, nullptr};
    // fp32 negabinary: the levels decoded by one multi-level launch
    ChunkSeg* dseg = nullptr;
    int dseg_n = 0;
    uint64_t dseg_chunks = 0;
    // fp32 negabinary: every level encoded by one launch (per-level partial
    // error tables in lpartial)
    ChunkSeg* eseg = nullptr;
    uint64_t eseg_chunks = 0;
    double* lpartial = nullptr;
    uint8_t* pack_tmp = nullptr;
    // reconstructor fed from level files (reference on-disk format)
    bool from_files = false;
    std::vector<uint32_t> hsizes;                  // host copy of the plane sizes
    std::vector<uint8_t*> lfile;                   // grouped: level-file bytes as loaded
    std::vector<uint64_t> loaded, unpacked;        // bytes loaded / planes unpacked per level
    std::vector<uint8_t> header_done;
    // optional stage timing: CUDA events recorded on the launching stream
    bool timing = false;
    struct Pending { int id; cudaEvent_t a, b; };
    std::vector<Pending> pending;
    std::vector<cudaEvent_t> pool;
    double stage_ms[5 * 17] = {0};
    uint32_t stage_n[5 * 17] = {0};
    cudaEvent_t ev() {
        cudaEvent_t e;
        if (!pool.empty()) { e = pool.back(); pool.pop_back(); }
        else cudaEventCreate(&e);
        return e;
    }
    int collect() {
        for (auto& p : pending) {
            cudaError_t e = cudaEventSynchronize(p.b);
            if (e != cudaSuccess) return cuda_status(e, "cudaEventSynchronize");
            float ms = 0;
            cudaEventElapsedTime(&ms, p.a, p.b);
            stage_ms[p.id] += ms;
            stage_n[p.id] += 1;
            pool.push_back(p.a);
            pool.push_back(p.b);
        }
        pending.clear();
        return PRODM_OK;
    }
    ~prodm_mdr() {
        if (fstage) file_staging_free(fstage);
        for (auto& p : pending) { cudaEventDestroy(p.a); cudaEventDestroy(p.b); }
        for (auto e : pool) cudaEventDestroy(e);
        for (void* p : allocs) cudaFree(p);
        if (hmap) cudaFreeHost(hmap);
    }
    int alloc(void** p, size_t bytes) {
        if (bytes == 0) bytes = 256;
        cudaError_t e = cudaMalloc(p, bytes);
        if (e != cudaSuccess) return cuda_status(e, "cudaMalloc");
        allocs.push_back(*p);
        return PRODM_OK;
    }
};

namespace prodm {
namespace {

// stage ids: kind * 17 + level; kinds 0 decompose, 1 encode, 2 interpret,
// 3 decode, 4 recompose
struct Stage {
    prodm_mdr* h;
    int id;
    cudaEvent_t a = nullptr, b = nullptr;
    cudaStream_t st;
    bool capturing = false;
    Stage(prodm_mdr* h_, int kind, int level, cudaStream_t st_) : h(h_), id(kind * 17 + level), st(st_) {
        if (h->timing) {
            cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
            cudaStreamIsCapturing(st, &cs);
            capturing = cs == cudaStreamCaptureStatusActive;
            a = h->ev();
            b = h->ev();
            record(a);
        }
    }
    // inside a stream capture the records become external event nodes, which
    // every replay of the graph records and the host can time
    void record(cudaEvent_t e) {
        if (capturing) cudaEventRecordWithFlags(e, st, cudaEventRecordExternal);
        else cudaEventRecord(e, st);
    }
    ~Stage() {
        if (a) {
            record(b);
            h->pending.push_back({id, a, b});
        }
    }
};

// Levels decoded inside their recomposition (fp32 negabinary, hierarchical):
// the finest level and the next one down when its rows are plenty
// (kFusedLevels in all; a third level, 129^3 at 513^3, measured slower);
// returns the lowest such level, or L + 1 for none.
constexpr int kFusedLevels = 2;
int fused_from(const prodm_mdr* h) {
    const int L = h->g.L;
    if (!(h->nb && !h->orth && h->cfg.dtype == PRODM_F32 && L >= 1 && decode_recompose_nb32_ok(h->g.box[L])))
        return L + 1;
    int from = L;
    while (from - 1 >= 1 && L - (from - 1) < kFusedLevels && decode_recompose_nb32_ok(h->g.box[from - 1]) &&
           (uint64_t)h->g.box[from - 1].n[0] * h->g.box[from - 1].n[1] >= 4096)
        from--;
    return from;
}

int mdr_alloc_all(prodm_mdr* h) {
    const LevelGeom& g = h->g;
    const int L = g.L, B = h->B;
    const size_t es = h->es;
    const int dtype = h->cfg.dtype;
    int rc;
    uint64_t N = g.total;
    if ((rc = h->alloc(&h->coef, N * es))) return rc;
    // decoded levels: each level starts on a 16-byte boundary (vector stores)
    h->roff.assign(L + 2, 0);
    for (int l = 0; l <= L; l++) h->roff[l + 1] = (h->roff[l] + g.elems[l] + 16 / es - 1) / (16 / es) * (16 / es);
    if ((rc = h->alloc(&h->rcoef, h->roff[L + 1] * es))) return rc;
    uint64_t cb = L >= 1 ? g.box[L - 1].size() : 1;
    for (int i = 0; i < 2; i++) {
        if ((rc = h->alloc(&h->cbuf[i], cb * es))) return rc;
        if ((rc = h->alloc(&h->rbuf[i], cb * es))) return rc;
    }
    if (h->orth && L >= 1) {
        const Box& F = g.box[L];
        Box C{{coarse_len(F.n[0]), coarse_len(F.n[1]), coarse_len(F.n[2])}};
        if ((rc = h->alloc(&h->os.t1, (uint64_t)F.n[0] * F.n[1] * C.n[2] * es))) return rc;
        if ((rc = h->alloc(&h->os.t2, (uint64_t)F.n[0] * C.n[1] * C.n[2] * es))) return rc;
        if ((rc = h->alloc(&h->os.z, C.size() * es))) return rc;
        if (dtype == PRODM_F64) {
            std::vector<double> tab = build_tabs<double>(g, h->tab_off);
            if ((rc = h->alloc(&h->tabs, tab.size() * 8))) return rc;
            PRODM_CUDA(cudaMemcpy(h->tabs, tab.data(), tab.size() * 8, cudaMemcpyHostToDevice));
        } else {
            std::vector<float> tab = build_tabs<float>(g, h->tab_off);
            if ((rc = h->alloc(&h->tabs, tab.size() * 4))) return rc;
            PRODM_CUDA(cudaMemcpy(h->tabs, tab.data(), tab.size() * 4, cudaMemcpyHostToDevice));
        }
    }
    // streams (aligned layout)
    h->lvl_byte_off.assign(L + 2, 0);
    h->plane_cap.assign(L + 1, 0);
    h->nblocks.assign(L + 1, 0);
    h->rb_off.assign(L + 2, 0);
    h->co_off.assign(L + 2, 0);
    uint64_t maxch = 0;
    for (int l = 0; l <= L; l++) {
        uint64_t nbk = nblocks_of(dtype, g.elems[l]);
        h->nblocks[l] = nbk;
        // negabinary planes start on 16-byte boundaries (rows padded to a
        // multiple of 16 bytes) so that whole plane runs move with 16-byte
        // copies; the pad words are never part of a stream
        const uint64_t pw = 16 / es;
        // per-bit: B magnitude rows + sign row + unseen row of u32 group words
        h->plane_cap[l] = h->pb ? pb_row_words(g.elems[l]) : h->nb ? (nbk + pw - 1) / pw * pw : 2 * nbk;
        h->lvl_byte_off[l + 1] = h->lvl_byte_off[l] + (h->pb ? (uint64_t)(B + 2) * h->plane_cap[l] * 4
                                                             : (uint64_t)B * h->plane_cap[l] * es);
        h->rb_off[l + 1] = h->rb_off[l] + nbk;
        uint64_t nch = gr_nchunks(nbk);
        maxch = nch > maxch ? nch : maxch;
        h->co_off[l + 1] = h->co_off[l] + nch * B;
    }
    if ((rc = h->alloc((void**)&h->streams, h->lvl_byte_off[L + 1]))) return rc;
    if ((rc = h->alloc(&h->keys, (L + 1) * 8))) return rc;
    if ((rc = h->alloc(&h->bounds, (L + 1) * es))) return rc;
    if ((rc = h->alloc((void**)&h->sizes, (L + 1) * B * 4))) return rc;
    if ((rc = h->alloc((void**)&h->rsizes, (L + 1) * B * 4))) return rc;
    if ((rc = h->alloc((void**)&h->sqerr, (L + 1) * (B + 1) * 8))) return rc;
    if ((rc = h->alloc((void**)&h->maxerr, (L + 1) * (B + 1) * 8))) return rc;
    uint64_t parts = maxch > (uint64_t)kPartialSlots ? maxch : (uint64_t)kPartialSlots;
    if ((rc = h->alloc((void**)&h->partial, partial_bytes(parts, B)))) return rc;
    if ((rc = h->alloc((void**)&h->index, L + 1 + 15))) return rc;
    if ((rc = h->alloc((void**)&h->rsz, (L + 1) * 4))) return rc;
    if ((rc = h->alloc((void**)&h->kstatus, 16))) return rc;
    PRODM_CUDA(cudaMemset(h->kstatus, 0, 16));
    PRODM_CUDA(cudaHostAlloc((void**)&h->hmap, 128, cudaHostAllocMapped));
    PRODM_CUDA(cudaHostGetDevicePointer((void**)&h->dmap, h->hmap, 0));
    if ((rc = h->alloc((void**)&h->ndims_d, 4))) return rc;
    if ((rc = h->alloc((void**)&h->levels_d, 4))) return rc;
    PRODM_CUDA(cudaMemset(h->sqerr, 0, (L + 1) * (B + 1) * 8));
    PRODM_CUDA(cudaMemset(h->index, 0, L + 1));
    PRODM_CUDA(cudaMemcpy(h->ndims_d, &g.ndims, 4, cudaMemcpyHostToDevice));
    PRODM_CUDA(cudaMemcpy(h->levels_d, &L, 4, cudaMemcpyHostToDevice));
    if (h->nb) {
        std::vector<uint32_t> sz((L + 1) * B);
        for (int l = 0; l <= L; l++)
            for (int p = 0; p < B; p++) sz[l * B + p] = (uint32_t)(h->nblocks[l] * es);
        PRODM_CUDA(cudaMemcpy(h->sizes, sz.data(), sz.size() * 4, cudaMemcpyHostToDevice));
    } else if (h->pb) {
        if ((rc = h->alloc((void**)&h->pbcounts, (L + 1) * 64 * 4))) return rc;
        if ((rc = h->alloc((void**)&h->pbstatus, 16))) return rc;
    } else {
        if ((rc = h->alloc((void**)&h->rbs, h->rb_off[L + 1]))) return rc;
        if ((rc = h->alloc((void**)&h->chunk_words, maxch * B * 4))) return rc;
        if ((rc = h->alloc((void**)&h->chunk_off, h->co_off[L + 1] * 4))) return rc;
        if ((rc = h->alloc((void**)&h->plane_ptrs, (L + 1) * B * sizeof(void*)))) return rc;
        std::vector<void*> ptrs((L + 1) * B);
        for (int l = 0; l <= L; l++)
            for (int p = 0; p < B; p++)
                ptrs[l * B + p] = h->streams + h->lvl_byte_off[l] + (uint64_t)p * h->plane_cap[l] * es;
        PRODM_CUDA(cudaMemcpy(h->plane_ptrs, ptrs.data(), ptrs.size() * sizeof(void*), cudaMemcpyHostToDevice));
    }
    if (h->nb && dtype == PRODM_F32) {
        // every level not decoded inside its recomposition, as one segment
        // table (kDecodeChunkBlocks blocks per chunk)
        const int top = fused_from(h) - 1;
        std::vector<ChunkSeg> segs;
        uint64_t chunks = 0;
        for (int l = 0; l <= top; l++) {
            ChunkSeg q{};
            q.y = (float*)h->rcoef + h->roff[l];
            q.words = (uint32_t*)(h->streams + h->lvl_byte_off[l]);
            q.n = g.elems[l];
            q.nblocks = h->nblocks[l];
            q.stride = h->plane_cap[l];
            q.key = (const uint32_t*)h->keys + l;
            q.dnum = h->index + l;
            q.chunk_begin = chunks;
            chunks += (q.nblocks + kDecodeChunkBlocks - 1) / kDecodeChunkBlocks;
            segs.push_back(q);
        }
        if ((rc = h->alloc((void**)&h->dseg, segs.size() * sizeof(ChunkSeg)))) return rc;
        PRODM_CUDA(cudaMemcpy(h->dseg, segs.data(), segs.size() * sizeof(ChunkSeg), cudaMemcpyHostToDevice));
        h->dseg_n = (int)segs.size();
        h->dseg_chunks = chunks;
        // encode: every level, coefficients in, planes out
        std::vector<ChunkSeg> esegs;
        chunks = 0;
        for (int l = 0; l <= L; l++) {
            ChunkSeg q{};
            q.x = (const float*)h->coef + g.offset[l];
            q.words = (uint32_t*)(h->streams + h->lvl_byte_off[l]);
            q.n = g.elems[l];
            q.nblocks = h->nblocks[l];
            q.stride = h->plane_cap[l];
            q.key = (const uint32_t*)h->keys + l;
            q.chunk_begin = chunks;
            chunks += (q.nblocks + 255) / 256;
            esegs.push_back(q);
        }
        if ((rc = h->alloc((void**)&h->eseg, esegs.size() * sizeof(ChunkSeg)))) return rc;
        PRODM_CUDA(cudaMemcpy(h->eseg, esegs.data(), esegs.size() * sizeof(ChunkSeg), cudaMemcpyHostToDevice));
        h->eseg_chunks = chunks;
        if (h->sq) {
            const size_t rows = (size_t)(L + 1) * nb_encode_levels_grid(1);
            if ((rc = h->alloc((void**)&h->lpartial, rows * kErrRecWords * 8))) return rc;
        }
    }
    return PRODM_OK;
}

template <class T>
const T* level_tabs(prodm_mdr* h, int l, int d) {
    return (const T*)h->tabs + h->tab_off[l * 3 + d];
}

template <class T>
int mdr_refactor(prodm_mdr* h, const T* field, cudaStream_t st) {
    const LevelGeom& g = h->g;
    const int L = g.L, B = h->B;
    using K = typename KeyOf<T>::type;
    K* keys = (K*)h->keys;
    T* coef = (T*)h->coef;
    int rc;
    PRODM_CUDA(cudaMemsetAsync(h->keys, 0, (L + 1) * 8, st));
    if (L == 0) {
        PRODM_CUDA(cudaMemcpyAsync(coef, field, g.total * sizeof(T), cudaMemcpyDeviceToDevice, st));
        if ((rc = launch_maxabs<T>(coef, g.total, keys, st))) return rc;
    } else {
        for (int l = L; l >= 1; l--) {
            const Box& F = g.box[l];
            const Box& C = g.box[l - 1];
            const T* in = (l == L) ? field : (const T*)h->cbuf[(l + 1) & 1];
            T* cout = (l == 1) ? coef + g.offset[0] : (T*)h->cbuf[l & 1];
            Stage sg(h, 0, l, st);
            if ((rc = launch_decompose_level_packed<T>(in, (uint64_t)F.n[1] * F.n[2], F.n[2], F, C, coef + g.offset[l],
                                                       cout, nullptr, keys + l,
                                                       (l == 1 && !h->orth) ? (void*)keys : nullptr, st)))
                return rc;
            if (h->orth) {   // the correction reads the level's packed coefficients
                const T* tabs[3] = {level_tabs<T>(h, l, 0), level_tabs<T>(h, l, 1), level_tabs<T>(h, l, 2)};
                if ((rc = launch_l2_correction<T>(nullptr, F, (T*)h->os.t1, (T*)h->os.t2, (T*)h->os.z, tabs, st,
                                                  coef + g.offset[l], &C)))
                    return rc;
                if ((rc = launch_add_box<T>(cout, (uint64_t)C.n[1] * C.n[2], C.n[2], (T*)h->os.z, C, (T)1, st))) return rc;
            }
        }
        if (h->orth && (rc = launch_maxabs<T>(coef, g.elems[0], keys, st))) return rc;
    }
    if ((rc = launch_bounds_from_keys<T>(keys, L + 1, h->nb ? 1 : 0, (T*)h->bounds, st))) return rc;
    if (h->eseg && sizeof(T) == 4) {
        // fp32 negabinary: every level in one launch (timed as the finest level)
        Stage sg(h, 1, L, st);
        return launch_nb_encode_levels(h->eseg, L + 1, h->eseg_chunks, B, h->lpartial, (const uint32_t*)keys,
                                       h->sq ? h->sqerr : nullptr, st);
    }
    for (int l = 0; l <= L; l++) {
        const uint64_t n = g.elems[l];
        uint8_t* out = h->streams + h->lvl_byte_off[l];
        double* errs = h->sq ? h->sqerr + (uint64_t)l * (B + 1) : nullptr;
        Stage sg(h, 1, l, st);
        if (h->pb) {
            rc = launch_pb_encode<T>(coef + g.offset[l], n, keys + l, 0, B, (uint32_t*)out, h->plane_cap[l],
                                     h->pbcounts + l * 64, h->sizes + (uint64_t)l * B, st);
        } else if (h->nb) {
            rc = launch_nb_encode<T>(coef + g.offset[l], n, keys + l, 0, B, out, h->plane_cap[l], h->partial, errs, st);
        } else {
            rc = launch_gr_encode<T>(coef + g.offset[l], n, keys + l, 0, B, h->rbs + h->rb_off[l], h->chunk_words,
                                     h->chunk_off + h->co_off[l], h->sizes + (uint64_t)l * B, out, h->plane_cap[l],
                                     h->partial, errs, st);
        }
        if (rc) return rc;
    }
    return PRODM_OK;
}

template <class T>
int mdr_decode_recompose(prodm_mdr* h, T* out, cudaStream_t st) {
    const LevelGeom& g = h->g;
    const int L = g.L, B = h->B;
    using K = typename KeyOf<T>::type;
    K* keys = (K*)h->keys;
    T* rcoef = (T*)h->rcoef;
    int rc;
    // finest level: fused decode + recompose where the layout allows it
    const int ffrom = fused_from(h);
    if (h->dseg && sizeof(T) == 4) {
        // fp32 negabinary: every other level in one launch (timed as level 0)
        Stage sg(h, 3, 0, st);
        if ((rc = launch_nb_decode_levels(h->dseg, h->dseg_n, h->dseg_chunks, st, true))) return rc;
    }
    for (int l = 0; l <= L; l++) {
        if (l >= ffrom || (h->dseg && sizeof(T) == 4)) continue;
        const uint64_t n = g.elems[l];
        Stage sg(h, 3, l, st);
        if (h->pb) {
            const uint32_t* rows = (const uint32_t*)(h->streams + h->lvl_byte_off[l]);
            rc = launch_pb_decode<T>(rows, h->plane_cap[l], n, keys + l, 0, B, 0, 0, h->index + l,
                                     rows + (uint64_t)B * h->plane_cap[l], nullptr, rcoef + h->roff[l], st);
        } else if (h->nb) {
            rc = launch_nb_decode<T>(h->streams + h->lvl_byte_off[l], h->plane_cap[l], n, keys + l, 0, 0, 0,
                                     h->index + l, rcoef + h->roff[l], st);
        } else {
            rc = launch_gr_decode<T>((const void* const*)(h->plane_ptrs + (uint64_t)l * B), n, keys + l, 0, B, 0, 0,
                                     h->index + l, h->rbs + h->rb_off[l], h->chunk_off + h->co_off[l], nullptr,
                                     rcoef + h->roff[l], st);
        }
        if (rc) return rc;
    }
    if (L == 0) {
        PRODM_CUDA(cudaMemcpyAsync(out, rcoef, g.total * sizeof(T), cudaMemcpyDeviceToDevice, st));
        return PRODM_OK;
    }
    for (int l = 1; l <= L; l++) {
        const Box& F = g.box[l];
        const Box& C = g.box[l - 1];
        T* cin = (l == 1) ? rcoef + h->roff[0] : (T*)h->rbuf[(l - 1) & 1];
        T* o = (l == L) ? out : (T*)h->rbuf[l & 1];
        Stage sg(h, 4, l, st);
        if (l >= ffrom) {
            if ((rc = launch_decode_recompose_nb32(h->streams + h->lvl_byte_off[l], h->plane_cap[l], B,
                                                   h->nblocks[l], keys + l, h->index + l, (const float*)cin, F, C,
                                                   (float*)o, (uint64_t)F.n[1] * F.n[2], F.n[2], h->kstatus, st,
                                                   true)))
                return rc;
            continue;
        }
        if (h->orth) {
            const T* tabs[3] = {level_tabs<T>(h, l, 0), level_tabs<T>(h, l, 1), level_tabs<T>(h, l, 2)};
            if ((rc = launch_l2_correction<T>(nullptr, F, (T*)h->os.t1, (T*)h->os.t2, (T*)h->os.z, tabs, st,
                                              rcoef + h->roff[l], &C)))
                return rc;
            if ((rc = launch_add_box<T>(cin, (uint64_t)C.n[1] * C.n[2], C.n[2], (T*)h->os.z, C, (T)-1, st))) return rc;
        }
        if ((rc = launch_recompose_level_packed<T>(cin, rcoef + h->roff[l], F, C, o, (uint64_t)F.n[1] * F.n[2], F.n[2],
                                                   st, true)))
            return rc;
    }
    return PRODM_OK;
}

template <class T>
int mdr_interpret(prodm_mdr* h, double tol, int interp, int est, double s, cudaStream_t st) {
    const int L = h->g.L, B = h->B;
    int rc;
    const double* errs;
    if (est == PRODM_EST_MAX_HB || est == PRODM_EST_MAX_OB) {
        if ((rc = launch_max_collect<T>((const T*)h->bounds, L + 1, B, h->maxerr, st))) return rc;
        errs = h->maxerr;
    } else {
        if (!h->sq) return fail(PRODM_EINVAL, "squared-error estimators need collector == PRODM_COLLECT_SQUARED");
        errs = h->sqerr;
    }
    Stage sg(h, 2, 0, st);
    // right after a reconstruction (whose kernels write none of the tables
    // and read the plane counts), the interpreter may tabulate before it waits
    const bool early = h->after_reconstruct;
    h->after_reconstruct = false;
    return launch_interpret<T>(1, interp, est, h->ndims_d, h->levels_d, s, B, h->sizes, 0, errs, 0, nullptr, tol,
                               h->index, 0, h->rsz, st, true, early);
}

// grouped levels loaded from files: header -> rb + chunk offsets, then the
// planes completely inside the loaded prefix -> aligned layout
// per-bit levels loaded from files: parse the planes that lie completely
// inside the loaded prefix and are not parsed yet into the level's rows
int pb_parse_loaded(prodm_mdr* h, int l, cudaStream_t st) {
    const int B = h->B;
    const uint64_t n = h->g.elems[l], rw = h->plane_cap[l];
    uint32_t* rows = (uint32_t*)(h->streams + h->lvl_byte_off[l]);
    int rc;
    if (!h->header_done[l]) {
        if ((rc = launch_pb_init_unseen(rows + (uint64_t)(B + 1) * rw, rows + (uint64_t)B * rw, n, st))) return rc;
        h->header_done[l] = 1;
    }
    uint64_t off = 0;
    int complete = 0;
    for (int p = 0; p < B; p++) {
        off += h->hsizes[l * B + p];
        if (off <= h->loaded[l]) complete = p + 1;
        else break;
    }
    const int first = (int)h->unpacked[l];
    if (complete <= first) return PRODM_OK;
    const int num = complete - first;
    std::vector<uint64_t> hv(2 * num);
    uint64_t o = 0;
    for (int p = 0; p < first; p++) o += h->hsizes[l * B + p];
    for (int i = 0; i < num; i++) {
        const uint64_t sz = h->hsizes[l * B + first + i];
        if (sz == 0 || sz % 8) return fail(PRODM_ECORRUPT, "load: per-bit stream size not a positive multiple of 8");
        hv[i] = (uint64_t)(uintptr_t)(h->lfile[l] + o);
        hv[num + i] = sz / 8;
        o += sz;
    }
    uint64_t* dv;   // plane pointers, word counts, then the parse pipeline's scratch
    const size_t head = (hv.size() * 8 + 255) / 256 * 256;
    PRODM_CUDA(cudaMallocAsync((void**)&dv, head + pb_parse_scratch_bytes(num), st));
    PRODM_CUDA(cudaMemcpyAsync(dv, hv.data(), hv.size() * 8, cudaMemcpyHostToDevice, st));
    PRODM_CUDA(cudaMemsetAsync(h->pbstatus, 0, 4, st));
    rc = launch_pb_parse((const uint64_t* const*)dv, dv + num, first, num, n, rows, rw, rows + (uint64_t)(B + 1) * rw,
                         rows + (uint64_t)B * rw, (uint8_t*)dv + head, h->pbstatus, st);
    int hstat = 0;
    if (!rc) {
        cudaError_t e = cudaMemcpyAsync(&hstat, h->pbstatus, 4, cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) rc = cuda_status(e, "per-bit load");
    }
    cudaFreeAsync(dv, st);
    if (rc) return rc;
    if (hstat == PRODM_ETIMEOUT) return fail(PRODM_ETIMEOUT, "load: the per-bit parse pipeline stalled");
    if (hstat) return fail(PRODM_ECORRUPT, "load: a per-bit stream does not end where its size says");
    h->unpacked[l] = complete;
    return PRODM_OK;
}

int mdr_unpack_loaded(prodm_mdr* h, cudaStream_t st) {
    const int L = h->g.L, B = h->B;
    const int wb = (int)h->es;
    int rc;
    for (int l = 0; l <= L; l++) {
        if (!h->lfile[l]) continue;
        if (h->pb) {
            if ((rc = pb_parse_loaded(h, l, st))) return rc;
            continue;
        }
        const uint64_t nbk = h->nblocks[l];
        const uint64_t hdr = 4 + nbk;
        if (!h->header_done[l]) {
            if (h->loaded[l] < hdr) continue;
            PRODM_CUDA(cudaMemcpyAsync(h->rbs + h->rb_off[l], h->lfile[l] + 4, nbk, cudaMemcpyDeviceToDevice, st));
            if ((rc = launch_chunk_words_from_rb(h->rbs + h->rb_off[l], nbk, B, h->chunk_words, st))) return rc;
            if ((rc = launch_gr_scan_only(h->chunk_words, gr_nchunks(nbk), B, nbk, wb, h->chunk_off + h->co_off[l],
                                          (uint32_t*)h->partial, st)))
                return rc;
            h->header_done[l] = 1;
        }
        // planes fully loaded
        uint64_t off = 0;
        int complete = 0;
        for (int p = 0; p < B; p++) {
            off += h->hsizes[l * B + p];
            if (off <= h->loaded[l]) complete = p + 1;
            else break;
        }
        int first = (int)h->unpacked[l];
        if (complete <= first) continue;
        int num = complete - first;
        std::vector<uint64_t> hostv(3 * num);
        uint64_t o = 0;
        for (int p = 0; p < first; p++) o += h->hsizes[l * B + p];
        uint64_t maxw = 0;
        for (int i = 0; i < num; i++) {
            int p = first + i;
            uint64_t skip = p == 0 ? hdr : 0;
            hostv[i] = o + skip;
            hostv[num + i] = (h->hsizes[l * B + p] - skip) / h->es;
            hostv[2 * num + i] = (uint64_t)(uintptr_t)(h->streams + h->lvl_byte_off[l] + (uint64_t)p * h->plane_cap[l] * h->es);
            maxw = hostv[num + i] > maxw ? hostv[num + i] : maxw;
            o += h->hsizes[l * B + p];
        }
        uint64_t* dv;
        PRODM_CUDA(cudaMallocAsync((void**)&dv, hostv.size() * 8, st));
        PRODM_CUDA(cudaMemcpyAsync(dv, hostv.data(), hostv.size() * 8, cudaMemcpyHostToDevice, st));
        PRODM_CUDA(cudaStreamSynchronize(st));
        rc = launch_unpack_planes(h->lfile[l], dv, dv + num, num, wb, (void* const*)(dv + 2 * num), maxw, st);
        cudaFreeAsync(dv, st);
        if (rc) return rc;
        h->unpacked[l] = complete;
    }
    return PRODM_OK;
}

int mdr_load_level(prodm_mdr* h, int l, const void* src, uint64_t off, uint64_t bytes, int host, cudaStream_t st);

// lossless stage: stored level bytes as they arrive
int mdr_ll_load(prodm_mdr* h, int l, const void* src, uint64_t off, uint64_t bytes, int host, cudaStream_t st) {
    const int B = h->B;
    uint64_t total = 0;
    for (int p = 0; p < B; p++) total += h->ll_stored[l * B + p];
    if (off + bytes > total) return fail(PRODM_EINVAL, "load_level: range beyond the level file");
    if (bytes == 0) return PRODM_OK;
    if (h->ll_zstd) {   // zstd planes are expanded on the host
        std::vector<uint8_t>& hb = h->ll_hbuf[l];
        if (hb.size() < total) hb.resize(total);
        if (host) {
            memcpy(hb.data() + off, src, bytes);
        } else {
            PRODM_CUDA(cudaMemcpyAsync(hb.data() + off, src, bytes, cudaMemcpyDeviceToHost, st));
            PRODM_CUDA(cudaStreamSynchronize(st));
        }
        if (off + bytes > h->ll_cloaded[l]) h->ll_cloaded[l] = off + bytes;
        return PRODM_OK;
    }
    if (!h->ll_cbuf[l]) {
        int rc = h->alloc((void**)&h->ll_cbuf[l], total);
        if (rc) return rc;
    }
    PRODM_CUDA(cudaMemcpyAsync(h->ll_cbuf[l] + off, src, bytes, host ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice,
                               st));
    if (off + bytes > h->ll_cloaded[l]) h->ll_cloaded[l] = off + bytes;
    return PRODM_OK;
}

// stored planes completely loaded and not expanded yet -> raw plane bytes
// (decompressed where the stage compressed them) -> the raw loading path
int mdr_ll_expand_zstd(prodm_mdr* h, cudaStream_t st) {
    const int L = h->g.L, B = h->B;
    for (int l = 0; l <= L; l++) {
        const std::vector<uint8_t>& hb = h->ll_hbuf[l];
        if (hb.empty()) continue;
        uint64_t off = 0, soff = 0;
        int complete = 0;
        for (int p = 0; p < B; p++) {
            off += h->ll_stored[l * B + p];
            if (off <= h->ll_cloaded[l]) complete = p + 1;
            else break;
        }
        const int first = h->ll_expanded[l];
        if (complete <= first) continue;
        for (int p = 0; p < first; p++) soff += h->ll_stored[l * B + p];
        const uint64_t cap = encode_bound(h->cfg.encoder, h->cfg.dtype, h->g.elems[l], B);
        std::vector<uint8_t> raw;
        for (int p = first; p < complete; p++) {
            const uint32_t sz = h->ll_stored[l * B + p];
            const size_t at = raw.size();
            if (h->ll_flags[(size_t)l * B + p]) {
                int rc = zstd_expand_plane(hb.data() + soff, sz, cap, raw);
                if (rc) return rc;
            } else {
                raw.insert(raw.end(), hb.data() + soff, hb.data() + soff + sz);
            }
            h->hsizes[l * B + p] = (uint32_t)(raw.size() - at);
            soff += sz;
        }
        if (!raw.empty()) {
            int rc = mdr_load_level(h, l, raw.data(), h->ll_rawoff[l], raw.size(), 1, st);
            if (!rc) {
                cudaError_t e = cudaStreamSynchronize(st);   // raw is pageable host memory
                if (e != cudaSuccess) rc = cuda_status(e, "zstd plane upload");
            }
            if (rc) return rc;
        }
        h->ll_rawoff[l] += raw.size();
        h->ll_expanded[l] = complete;
    }
    return PRODM_OK;
}

int mdr_ll_expand(prodm_mdr* h, cudaStream_t st) {
    const int L = h->g.L, B = h->B;
    if (h->ll_zstd) return mdr_ll_expand_zstd(h, st);
    for (int l = 0; l <= L; l++) {
        if (!h->ll_cbuf[l]) continue;
        uint64_t off = 0, soff = 0;
        int complete = 0;
        for (int p = 0; p < B; p++) {
            off += h->ll_stored[l * B + p];
            if (off <= h->ll_cloaded[l]) complete = p + 1;
            else break;
        }
        const int first = h->ll_expanded[l];
        if (complete <= first) continue;
        const int num = complete - first;
        for (int p = 0; p < first; p++) soff += h->ll_stored[l * B + p];
        const uint64_t cap = encode_bound(h->cfg.encoder, h->cfg.dtype, h->g.elems[l], B);
        uint8_t* raw;
        PRODM_CUDA(cudaMallocAsync((void**)&raw, cap + 256, st));
        std::vector<uint32_t> rsz(num);
        int rc = ll_decompress_planes(h->ll_cbuf[l] + soff, h->ll_stored.data() + l * B + first,
                                      h->ll_flags.data() + (size_t)l * B + first, num, raw, cap, rsz.data(), st);
        uint64_t rbytes = 0;
        if (!rc) {
            for (int i = 0; i < num; i++) {
                h->hsizes[l * B + first + i] = rsz[i];
                rbytes += rsz[i];
            }
            rc = mdr_load_level(h, l, raw, h->ll_rawoff[l], rbytes, 0, st);
        }
        cudaFreeAsync(raw, st);
        if (rc) return rc;
        h->ll_rawoff[l] += rbytes;
        h->ll_expanded[l] = complete;
    }
    return PRODM_OK;
}

template <class T>
int mdr_reconstruct(prodm_mdr* h, T* out, cudaStream_t st) {
    int rc;
    h->after_reconstruct = false;
    if (h->from_files && h->ll_latter >= 0 && (rc = mdr_ll_expand(h, st))) return rc;
    if (h->from_files && !h->nb && (rc = mdr_unpack_loaded(h, st))) return rc;
    if ((rc = mdr_decode_recompose<T>(h, out, st))) return rc;
    h->after_reconstruct = true;
    return PRODM_OK;
}

template <class T>
int mdr_retrieve(prodm_mdr* h, double tol, int interp, int est, double s, T* out, cudaStream_t st) {
    int rc = mdr_interpret<T>(h, tol, interp, est, s, st);
    if (rc) return rc;
    return mdr_reconstruct<T>(h, out, st);
}

template <class T>
int mdr_load_metadata(prodm_mdr* h, const uint8_t* buf, size_t len, cudaStream_t st) {
    const int L = h->g.L, B = h->B, nl = L + 1, nd = h->g.ndims;
    const uint8_t* p = buf;
    const uint8_t* end = buf + len;
    auto need = [&](size_t k) { return (size_t)(end - p) >= k; };
    if (!need(1) || *p++ != nd) return fail(PRODM_ECORRUPT, "metadata: dimension count mismatch");
    if (!need(4 * nd)) return fail(PRODM_ECORRUPT, "metadata truncated");
    for (int d = 0; d < nd; d++) {
        uint32_t v;
        memcpy(&v, p, 4);
        p += 4;
        if (v != h->g.dims[d]) return fail(PRODM_ECORRUPT, "metadata: dims mismatch");
    }
    if (!need(1) || *p++ != nl) return fail(PRODM_ECORRUPT, "metadata: level count mismatch");
    if (!need(nl * sizeof(T))) return fail(PRODM_ECORRUPT, "metadata truncated");
    std::vector<T> bounds(nl);
    memcpy(bounds.data(), p, nl * sizeof(T));
    p += nl * sizeof(T);
    h->hsizes.assign(nl * B, 0);
    for (int l = 0; l < nl; l++) {
        uint32_t c;
        if (!need(4)) return fail(PRODM_ECORRUPT, "metadata truncated");
        memcpy(&c, p, 4);
        p += 4;
        if ((int)c != B) return fail(PRODM_ECORRUPT, "metadata: bitplane count mismatch");
        if (!need(4 * B)) return fail(PRODM_ECORRUPT, "metadata truncated");
        memcpy(h->hsizes.data() + l * B, p, 4 * B);
        p += 4 * B;
    }
    if (!need(nl + 4 * nl + 1)) return fail(PRODM_ECORRUPT, "metadata truncated");
    std::vector<uint8_t> stops(p, p + nl);
    bool any_stop = false;
    for (int l = 0; l < nl; l++) any_stop |= stops[l] != 0;
    p += nl + 4 * nl;
    uint8_t negab = *p++;
    if ((negab != 0) != h->nb) return fail(PRODM_ECORRUPT, "metadata: encoder kind mismatch");
    std::vector<double> sq(nl * (B + 1), 0.0);
    if (need(8) && memcmp(p, "SQER", 4) == 0) {
        uint32_t c;
        memcpy(&c, p + 4, 4);
        p += 8;
        if ((int)c != B + 1 || !need(nl * (B + 1) * 8)) return fail(PRODM_ECORRUPT, "metadata: bad error-table extension");
        memcpy(sq.data(), p, nl * (B + 1) * 8);
        p += nl * (B + 1) * 8;
    }
    int latter = -1;
    bool zstd = false;
    if (need(8) && memcmp(p, "ZCB1", 4) == 0) {
        uint32_t lt;
        memcpy(&lt, p + 4, 4);
        if (lt > 255) return fail(PRODM_ECORRUPT, "metadata: bad lossless-stage extension");
        latter = (int)lt;
    } else if (any_stop) {
        // stopping indices without this library's marker: the reference's
        // AdaptiveLevelCompressor wrote the levels with zstd; its latter index
        // is not in the metadata (the handle's, 26 unless set)
        if (!zstd_available())
            return fail(PRODM_EUNSUPPORTED, "metadata: levels compressed by the reference's zstd stage, and "
                                            "libzstd.so.1 could not be opened");
        latter = h->zstd_latter;
        zstd = true;
    }
    // device state: sizes, bounds, level max keys (exponents) and error tables
    using K = typename KeyOf<T>::type;
    std::vector<K> keys(nl);
    for (int l = 0; l < nl; l++) {
        T m = h->nb ? bounds[l] / (T)4 : bounds[l];
        memcpy(&keys[l], &m, sizeof(T));
    }
    std::vector<uint8_t> kb(nl * 8, 0);
    memcpy(kb.data(), keys.data(), nl * sizeof(K));
    PRODM_CUDA(cudaMemcpyAsync(h->sizes, h->hsizes.data(), nl * B * 4, cudaMemcpyHostToDevice, st));
    PRODM_CUDA(cudaMemcpyAsync(h->bounds, bounds.data(), nl * sizeof(T), cudaMemcpyHostToDevice, st));
    PRODM_CUDA(cudaMemcpyAsync(h->keys, kb.data(), nl * sizeof(K), cudaMemcpyHostToDevice, st));
    PRODM_CUDA(cudaMemcpyAsync(h->sqerr, sq.data(), sq.size() * 8, cudaMemcpyHostToDevice, st));
    PRODM_CUDA(cudaMemsetAsync(h->index, 0, nl, st));
    PRODM_CUDA(cudaStreamSynchronize(st));
    h->from_files = true;
    h->hsz_valid = false;
    h->loaded.assign(nl, 0);
    h->unpacked.assign(nl, 0);
    h->header_done.assign(nl, 0);
    h->ll_latter = latter;
    if (latter >= 0) {
        // stored sizes stay the cost model; the raw sizes of compressed planes
        // become known as the planes are expanded (until then a placeholder
        // larger than any plane, so that no raw path counts them as loaded)
        h->ll_stop = stops;
        h->ll_stored = h->hsizes;
        h->ll_flags.assign((size_t)nl * B, 0);
        for (int l = 0; l < nl; l++)
            for (int q = 0; q < B; q++) {
                const bool c = q <= stops[l] || q >= latter;   // AdaptiveLevelCompressor.hpp:43-52
                h->ll_flags[(size_t)l * B + q] = c;
                if (c) h->hsizes[l * B + q] = h->nb ? (uint32_t)(h->nblocks[l] * h->es) : 0x3fffffffu;
            }
        h->ll_cloaded.assign(nl, 0);
        h->ll_rawoff.assign(nl, 0);
        h->ll_expanded.assign(nl, 0);
        if (h->ll_cbuf.empty()) h->ll_cbuf.assign(nl, nullptr);
    }
    h->ll_zstd = zstd;
    h->ll_hbuf.assign(zstd ? nl : 0, std::vector<uint8_t>());
    if (h->lfile.empty()) h->lfile.assign(nl, nullptr);
    return PRODM_OK;
}

int mdr_load_level(prodm_mdr* h, int l, const void* src, uint64_t off, uint64_t bytes, int host, cudaStream_t st) {
    const int B = h->B;
    if (!h->from_files) return fail(PRODM_EINVAL, "load_level: load the metadata first");
    uint64_t total = 0;
    for (int p = 0; p < B; p++) total += h->hsizes[l * B + p];
    // with the lossless stage the raw sizes of planes not yet expanded are
    // unknown: the raw level file is bounded by the encoder's bound
    if (h->ll_latter >= 0) total = encode_bound(h->cfg.encoder, h->cfg.dtype, h->g.elems[l], B);
    if (off + bytes > total) return fail(PRODM_EINVAL, "load_level: range beyond the level file");
    if (bytes == 0) return PRODM_OK;
    cudaMemcpyKind kind = host ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice;
    if (h->nb) {   // level-file bytes [off, off + bytes) -> padded plane rows
        const uint64_t row = h->nblocks[l] * h->es, pitch = h->plane_cap[l] * h->es;
        uint64_t pos = off, done = 0;
        while (done < bytes) {
            const uint64_t p = pos / row, within = pos - p * row;
            const uint64_t piece = std::min<uint64_t>(row - within, bytes - done);
            PRODM_CUDA(cudaMemcpyAsync(h->streams + h->lvl_byte_off[l] + p * pitch + within,
                                       (const uint8_t*)src + done, piece, kind, st));
            pos += piece;
            done += piece;
        }
    } else {
        if (!h->lfile[l]) {
            int rc = h->alloc((void**)&h->lfile[l], total);
            if (rc) return rc;
        }
        PRODM_CUDA(cudaMemcpyAsync(h->lfile[l] + off, src, bytes, kind, st));
    }
    if (off + bytes > h->loaded[l]) h->loaded[l] = off + bytes;
    return PRODM_OK;
}

}  // namespace
}  // namespace prodm

// ===========================================================================
// packed level coefficients <-> natural field, the pair behind the QoI
// gradient: forward = reposition every level + recompose
// (ComposedReconstructor.hpp:124-131 with MGARD.hpp:25-35; the orthogonal
// basis removes each level's L2 correction from its coarse box first),
// adjoint = its transpose. Workspace: two boxes of level L-1; orthogonal
// adds the Thomas tables, the correction's scratch boxes of level L and the
// adjoint's (boxes (n0, c1, c2), (n0, n1, c2), the level-L box, one coarse box).
namespace prodm {
void packed_pair_reserve(Workspace& ws, const LevelGeom& g, int basis, size_t es) {
    const int L = g.L;
    if (L == 0) return;
    const size_t cb = g.box[L - 1].size() * es;
    ws.reserve(cb);
    ws.reserve(cb);
    if (basis != PRODM_BASIS_ORTHOGONAL) return;
    const Box& F = g.box[L];
    const Box& C = g.box[L - 1];
    ws.reserve((tab_elems(g) + 1) * es);
    ws.reserve((uint64_t)F.n[0] * C.n[1] * C.n[2] * es);   // t2 / s_a
    ws.reserve((uint64_t)F.n[0] * F.n[1] * C.n[2] * es);   // t1 / s_b
    ws.reserve(F.size() * es);                               // s_w
    ws.reserve(C.size() * es);                               // z / s_u
}

template <class T>
int packed_pair_impl(const T* in, int ndims, const uint32_t* dims, int L, T* out, bool adjoint, int basis, void* wsp,
                     size_t wsb, cudaStream_t st) {
    LevelGeom g;
    int rc;
    if ((rc = make_geom(ndims, dims, L, g))) return rc;
    if (L > max_level(ndims, dims)) return fail(PRODM_EINVAL, "target level above the maximum for these dims");
    if (basis != PRODM_BASIS_HIERARCHICAL && basis != PRODM_BASIS_ORTHOGONAL) return fail(PRODM_EINVAL, "unknown basis");
    if (L == 0) {
        PRODM_CUDA(cudaMemcpyAsync(out, in, g.total * sizeof(T), cudaMemcpyDeviceToDevice, st));
        return PRODM_OK;
    }
    const bool orth = basis == PRODM_BASIS_ORTHOGONAL;
    const size_t cb = g.box[L - 1].size() * sizeof(T);
    Workspace ws(wsp, wsb, st);
    packed_pair_reserve(ws, g, basis, sizeof(T));
    if ((rc = ws.commit())) return rc;
    T* buf[2] = {(T*)ws.take(cb), (T*)ws.take(cb)};
    T *dtab = nullptr, *s_a = nullptr, *s_b = nullptr, *s_w = nullptr, *s_u = nullptr;
    std::vector<size_t> toff;
    if (orth) {
        const Box& F = g.box[L];
        const Box& C = g.box[L - 1];
        std::vector<T> tab = build_tabs<T>(g, toff);
        dtab = (T*)ws.take((tab_elems(g) + 1) * sizeof(T));
        s_a = (T*)ws.take((uint64_t)F.n[0] * C.n[1] * C.n[2] * sizeof(T));
        s_b = (T*)ws.take((uint64_t)F.n[0] * F.n[1] * C.n[2] * sizeof(T));
        s_w = (T*)ws.take(F.size() * sizeof(T));
        s_u = (T*)ws.take(C.size() * sizeof(T));
        PRODM_CUDA(cudaMemcpyAsync(dtab, tab.data(), tab.size() * sizeof(T), cudaMemcpyHostToDevice, st));
        PRODM_CUDA(cudaStreamSynchronize(st));   // host table lifetime
    }
    auto tabs_of = [&](int l, const T* (&t)[3]) {
        for (int d = 0; d < 3; d++) t[d] = dtab + toff[l * 3 + d];
    };
    if (!adjoint) {
        for (int l = 1; l <= L; l++) {
            const Box& F = g.box[l];
            const Box& C = g.box[l - 1];
            const T* cin = (l == 1) ? in + g.offset[0] : buf[(l - 1) & 1];
            T* o = (l == L) ? out : buf[l & 1];
            if (orth) {   // coarse box minus the level's correction (a copy of level 0 first)
                if (l == 1) {
                    PRODM_CUDA(cudaMemcpyAsync(buf[0], cin, C.size() * sizeof(T), cudaMemcpyDeviceToDevice, st));
                    cin = buf[0];
                }
                const T* tabs[3];
                tabs_of(l, tabs);
                if ((rc = launch_l2_correction<T>(nullptr, F, s_b, s_a, s_u, tabs, st, in + g.offset[l], &C))) return rc;
                if ((rc = launch_add_box<T>(const_cast<T*>(cin), (uint64_t)C.n[1] * C.n[2], C.n[2], s_u, C, (T)-1, st)))
                    return rc;
            }
            if ((rc = launch_recompose_level_packed<T>(cin, in + g.offset[l], F, C, o, (uint64_t)F.n[1] * F.n[2], F.n[2],
                                                       st)))
                return rc;
        }
        return PRODM_OK;
    }
    const T* gin = in;
    for (int l = L; l >= 1; l--) {
        T* gout = (l == 1) ? out + g.offset[0] : buf[l & 1];
        if (orth) {
            const T* tabs[3];
            tabs_of(l, tabs);
            rc = launch_recompose_adjoint_level_orth<T>(gin, g.box[l], g.box[l - 1], out + g.offset[l], gout, tabs, s_a,
                                                        s_b, s_w, s_u, st);
        } else {
            rc = launch_recompose_adjoint_level<T>(gin, g.box[l], g.box[l - 1], out + g.offset[l], gout, st);
        }
        if (rc) return rc;
        gin = gout;
    }
    return PRODM_OK;
}
}  // namespace prodm

// extern "C"
// ===========================================================================
#define DISPATCH(dtype, FN, ...) ((dtype) == PRODM_F64 ? FN<double>(__VA_ARGS__) : FN<float>(__VA_ARGS__))

extern "C" {

const char* prodm_last_error_string(void) { return prodm::g_err.c_str(); }
int prodm_version(void) { return 100; }

int prodm_max_level(int ndims, const uint32_t* dims, int* out) {
    if (!dims || !out || ndims < 1 || ndims > 3) return fail(PRODM_EINVAL, "prodm_max_level: bad arguments");
    *out = max_level(ndims, dims);
    return PRODM_OK;
}

int prodm_level_dims(int ndims, const uint32_t* dims, int L, uint32_t* out_dims, uint64_t* out_elems) {
    LevelGeom g;
    int rc = make_geom(ndims, dims, L, g);
    if (rc) return rc;
    for (int l = 0; l <= L; l++) {
        if (out_dims)
            for (int d = 0; d < ndims; d++) out_dims[l * ndims + d] = g.box[l].n[3 - ndims + d];
        if (out_elems) out_elems[l] = g.elems[l];
    }
    return PRODM_OK;
}

int prodm_decompose_workspace(int dtype, int ndims, const uint32_t* dims, uint32_t L, int basis, size_t* bytes) {
    int rc = check_dtype(dtype);
    if (rc) return rc;
    if (!bytes) return fail(PRODM_EINVAL, "bytes is NULL");
    return decompose_ws_bytes(dtype, ndims, dims, (int)L, basis, bytes);
}

int prodm_decompose(int dtype, void* d, int ndims, const uint32_t* dims, uint32_t L, const uint32_t* strides, int basis,
                    void* ws, size_t wsb, void* stream) {
    int rc = check_dtype(dtype);
    if (rc) return rc;
    if (!d || !dims) return fail(PRODM_EINVAL, "prodm_decompose: NULL pointer");
    if (dtype == PRODM_F64)
        return decompose_impl<double>((double*)d, ndims, dims, (int)L, strides, basis, ws, wsb, (cudaStream_t)stream, false);
    return decompose_impl<float>((float*)d, ndims, dims, (int)L, strides, basis, ws, wsb, (cudaStream_t)stream, false);
}

int prodm_recompose(int dtype, void* d, int ndims, const uint32_t* dims, uint32_t L, const uint32_t* strides, int basis,
                    void* ws, size_t wsb, void* stream) {
    int rc = check_dtype(dtype);
    if (rc) return rc;
    if (!d || !dims) return fail(PRODM_EINVAL, "prodm_recompose: NULL pointer");
    if (dtype == PRODM_F64)
        return decompose_impl<double>((double*)d, ndims, dims, (int)L, strides, basis, ws, wsb, (cudaStream_t)stream, true);
    return decompose_impl<float>((float*)d, ndims, dims, (int)L, strides, basis, ws, wsb, (cudaStream_t)stream, true);
}

static int interleave_common(int dtype, void* data, int ndims, const uint32_t* dims, const uint32_t* fine,
                             const uint32_t* coarse, void* buf, const uint32_t* strides, void* stream, bool gather) {
    int rc = check_dtype(dtype);
    if (rc) return rc;
    if (!data || !dims || !fine || !coarse || !buf) return fail(PRODM_EINVAL, "interleave: NULL pointer");
    if (ndims < 1 || ndims > 3) return fail(PRODM_EINVAL, "interleave: ndims must be 1, 2 or 3");
    uint64_t s0, s1;
    if ((rc = view_strides(ndims, dims, strides, s0, s1))) return rc;
    Box F, C;
    bool allz = true;
    for (int d = 0; d < ndims; d++) allz &= coarse[d] == 0;
    for (int i = 0; i < 3; i++) {
        int k = i - (3 - ndims);
        F.n[i] = k < 0 ? 1 : fine[k];
        C.n[i] = allz ? 0 : (k < 0 ? 1 : coarse[k]);
        if (k >= 0 && (fine[k] > dims[k] || coarse[k] > fine[k]))
            return fail(PRODM_EINVAL, "interleave: boxes must nest inside dims");
    }
    if (dtype == PRODM_F64)
        return launch_interleave<double>((double*)data, s0, s1, F, C, (double*)buf, gather, (cudaStream_t)stream);
    return launch_interleave<float>((float*)data, s0, s1, F, C, (float*)buf, gather, (cudaStream_t)stream);
}

int prodm_interleave(int dtype, const void* d_data, int ndims, const uint32_t* dims, const uint32_t* fine,
                     const uint32_t* coarse, void* d_buf, const uint32_t* strides, void* stream) {
    return interleave_common(dtype, (void*)d_data, ndims, dims, fine, coarse, d_buf, strides, stream, true);
}

int prodm_reposition(int dtype, const void* d_buf, int ndims, const uint32_t* dims, const uint32_t* fine,
                     const uint32_t* coarse, void* d_data, const uint32_t* strides, void* stream) {
    return interleave_common(dtype, d_data, ndims, dims, fine, coarse, (void*)d_buf, strides, stream, false);
}

int prodm_encode_bound(int enc, int dtype, uint64_t n, int B, uint64_t* out) {
    int rc = check_dtype(dtype);
    if (rc) return rc;
    if (!out) return fail(PRODM_EINVAL, "NULL output");
    *out = encode_bound(enc, dtype, n, B);
    return PRODM_OK;
}

int prodm_encode_workspace(int enc, int dtype, uint64_t n, int B, size_t* bytes) {
    int rc = check_dtype(dtype);
    if (rc) return rc;
    if (!bytes) return fail(PRODM_EINVAL, "NULL output");
    Workspace ws(nullptr, 0, 0);
    encode_reserve(ws, enc, dtype, n, B);
    *bytes = ws.needed();
    return PRODM_OK;
}

int prodm_encode(int enc, int dtype, const void* d, uint64_t n, int exp, int B, void* blob, uint64_t cap,
                 uint32_t* sizes, double* errs, void* ws, size_t wsb, void* stream) {
    int rc = check_dtype(dtype);
    if (rc) return rc;
    if (enc != PRODM_ENC_NEGABINARY && enc != PRODM_ENC_GROUPED && enc != PRODM_ENC_PERBIT)
        return fail(PRODM_EINVAL, "unknown encoder");
    if (!d || !blob || !sizes) return fail(PRODM_EINVAL, "prodm_encode: NULL pointer");
    if (dtype == PRODM_F64)
        return encode_impl<double>(enc, (const double*)d, n, exp, B, (uint8_t*)blob, cap, sizes, errs, ws, wsb,
                                   (cudaStream_t)stream);
    return encode_impl<float>(enc, (const float*)d, n, exp, B, (uint8_t*)blob, cap, sizes, errs, ws, wsb,
                              (cudaStream_t)stream);
}

int prodm_decoder_create(prodm_decoder** out, int enc, int dtype) {
    int rc = check_dtype(dtype);
    if (rc) return rc;
    if (!out) return fail(PRODM_EINVAL, "NULL output");
    if (enc != PRODM_ENC_NEGABINARY && enc != PRODM_ENC_GROUPED && enc != PRODM_ENC_PERBIT)
        return fail(PRODM_EINVAL, "unknown encoder");
    prodm_decoder* h = new prodm_decoder();
    h->enc = enc;
    h->dtype = dtype;
    *out = h;
    return PRODM_OK;
}

int prodm_progressive_decode(prodm_decoder* h, const void* blob, const uint32_t* hs, uint64_t n, int exp, int s, int num,
                             int level, int B, void* out, void* stream) {
    if (!h || !out || (num > 0 && (!blob || !hs))) return fail(PRODM_EINVAL, "prodm_progressive_decode: NULL pointer");
    if (level < 0 || level > 64) return fail(PRODM_EINVAL, "level out of range");
    if (h->dtype == PRODM_F64)
        return progressive_decode_impl<double>(h, (const uint8_t*)blob, hs, n, exp, s, num, level, B, (double*)out,
                                               (cudaStream_t)stream);
    return progressive_decode_impl<float>(h, (const uint8_t*)blob, hs, n, exp, s, num, level, B, (float*)out,
                                          (cudaStream_t)stream);
}

int prodm_decoder_destroy(prodm_decoder* h) {
    delete h;
    return PRODM_OK;
}

int prodm_collect_max(int dtype, double bound, int B, double* out) {
    int rc = check_dtype(dtype);
    if (rc) return rc;
    if (!out || B < 1) return fail(PRODM_EINVAL, "prodm_collect_max: bad arguments");
    int e = 0;
    if (dtype == PRODM_F32) std::frexp((float)bound, &e);
    else std::frexp(bound, &e);
    out[0] = dtype == PRODM_F32 ? (double)(float)bound : bound;
    double err = std::ldexp(1.0, e - 1);
    for (int i = 1; i <= B; i++) { out[i] = err; err /= 2; }
    return PRODM_OK;
}

int prodm_recompose_packed_basis_workspace(int dtype, int basis, int ndims, const uint32_t* dims, uint32_t L,
                                           size_t* bytes) {
    int rc = check_dtype(dtype);
    if (rc) return rc;
    if (!dims || !bytes) return fail(PRODM_EINVAL, "NULL pointer");
    if (basis != PRODM_BASIS_HIERARCHICAL && basis != PRODM_BASIS_ORTHOGONAL) return fail(PRODM_EINVAL, "unknown basis");
    LevelGeom g;
    if ((rc = make_geom(ndims, dims, (int)L, g))) return rc;
    Workspace ws(nullptr, 0, 0);
    packed_pair_reserve(ws, g, basis, esize(dtype));
    *bytes = ws.needed();
    return PRODM_OK;
}

int prodm_recompose_packed_workspace(int dtype, int ndims, const uint32_t* dims, uint32_t L, size_t* bytes) {
    return prodm_recompose_packed_basis_workspace(dtype, PRODM_BASIS_HIERARCHICAL, ndims, dims, L, bytes);
}

int prodm_recompose_packed_basis(int dtype, int basis, const void* d_coef, int ndims, const uint32_t* dims, uint32_t L,
                                 void* d_out, void* ws, size_t wsb, void* stream) {
    int rc = check_dtype(dtype);
    if (rc) return rc;
    if (!d_coef || !d_out || !dims) return fail(PRODM_EINVAL, "prodm_recompose_packed: NULL pointer");
    if (dtype == PRODM_F64)
        return packed_pair_impl<double>((const double*)d_coef, ndims, dims, (int)L, (double*)d_out, false, basis, ws,
                                        wsb, (cudaStream_t)stream);
    return packed_pair_impl<float>((const float*)d_coef, ndims, dims, (int)L, (float*)d_out, false, basis, ws, wsb,
                                   (cudaStream_t)stream);
}

int prodm_recompose_packed(int dtype, const void* d_coef, int ndims, const uint32_t* dims, uint32_t L, void* d_out,
                           void* ws, size_t wsb, void* stream) {
    return prodm_recompose_packed_basis(dtype, PRODM_BASIS_HIERARCHICAL, d_coef, ndims, dims, L, d_out, ws, wsb,
                                        stream);
}

int prodm_recompose_adjoint_basis(int dtype, int basis, const void* d_grad, int ndims, const uint32_t* dims,
                                  uint32_t L, void* d_grad_coef, void* ws, size_t wsb, void* stream) {
    int rc = check_dtype(dtype);
    if (rc) return rc;
    if (!d_grad || !d_grad_coef || !dims) return fail(PRODM_EINVAL, "prodm_recompose_adjoint: NULL pointer");
    if (dtype == PRODM_F64)
        return packed_pair_impl<double>((const double*)d_grad, ndims, dims, (int)L, (double*)d_grad_coef, true, basis,
                                        ws, wsb, (cudaStream_t)stream);
    return packed_pair_impl<float>((const float*)d_grad, ndims, dims, (int)L, (float*)d_grad_coef, true, basis, ws,
                                   wsb, (cudaStream_t)stream);
}

int prodm_recompose_adjoint(int dtype, const void* d_grad, int ndims, const uint32_t* dims, uint32_t L,
                            void* d_grad_coef, void* ws, size_t wsb, void* stream) {
    return prodm_recompose_adjoint_basis(dtype, PRODM_BASIS_HIERARCHICAL, d_grad, ndims, dims, L, d_grad_coef, ws, wsb,
                                         stream);
}

int prodm_collect_squared_workspace(int dtype, int B, size_t* bytes) {
    int rc = check_dtype(dtype);
    if (rc) return rc;
    if (!bytes) return fail(PRODM_EINVAL, "NULL output");
    *bytes = (size_t)kPartialSlots * (B + 1) * sizeof(double);
    return PRODM_OK;
}

int prodm_collect_squared(int dtype, const void* d, uint64_t n, int B, double maxv, double* out, void* wsp, size_t wsb,
                          void* stream) {
    int rc = check_dtype(dtype);
    if (rc) return rc;
    if (!d || !out) return fail(PRODM_EINVAL, "prodm_collect_squared: NULL pointer");
    if (B < 1 || B > (dtype == PRODM_F64 ? 64 : 32)) return fail(PRODM_EINVAL, "num_bitplanes out of range");
    cudaStream_t st = (cudaStream_t)stream;
    Workspace ws(wsp, wsb, st);
    ws.reserve((size_t)kPartialSlots * (B + 1) * sizeof(double));
    if ((rc = ws.commit())) return rc;
    double* partial = (double*)ws.take((size_t)kPartialSlots * (B + 1) * sizeof(double));
    if (dtype == PRODM_F64) return launch_sq_collect<double>((const double*)d, n, B, maxv, partial, out, st);
    return launch_sq_collect<float>((const float*)d, n, B, (float)maxv, partial, out, st);
}

int prodm_interpret(int interp, int est, int dtype, int ndims, int L, double s, int nl, int B, const uint32_t* d_sizes,
                    const double* d_errs, double tol, uint8_t* d_index, uint32_t* d_rsz, void* stream) {
    int rc = check_dtype(dtype);
    if (rc) return rc;
    if (interp < 0 || interp > 2 || est < 0 || est > 3) return fail(PRODM_EINVAL, "unknown interpreter or estimator");
    if (nl < 1 || nl > 17 || L < 0 || L > 16 || B < 1 || B > 64) return fail(PRODM_EINVAL, "prodm_interpret: sizes out of range");
    if (!d_sizes || !d_errs || !d_index || !d_rsz) return fail(PRODM_EINVAL, "prodm_interpret: NULL pointer");
    cudaStream_t st = (cudaStream_t)stream;
    int* p;
    PRODM_CUDA(cudaMallocAsync((void**)&p, 8, st));
    int hv[2] = {ndims, L};
    PRODM_CUDA(cudaMemcpyAsync(p, hv, 8, cudaMemcpyHostToDevice, st));
    if (dtype == PRODM_F64)
        rc = launch_interpret<double>(1, interp, est, p, p + 1, s, B, d_sizes, 0, d_errs, 0, nullptr, tol, d_index, 0,
                                      d_rsz, st);
    else
        rc = launch_interpret<float>(1, interp, est, p, p + 1, s, B, d_sizes, 0, d_errs, 0, nullptr, tol, d_index, 0,
                                     d_rsz, st);
    cudaError_t e = cudaStreamSynchronize(st);   // host array hv must outlive the copy
    cudaFreeAsync(p, st);
    if (rc) return rc;
    if (e != cudaSuccess) return cuda_status(e, "prodm_interpret");
    return PRODM_OK;
}

// ---------------------------------------------------------------------------
int prodm_mdr_create(prodm_mdr** out, const prodm_config* cfg) {
    if (!out || !cfg) return fail(PRODM_EINVAL, "prodm_mdr_create: NULL pointer");
    int rc = check_dtype(cfg->dtype);
    if (rc) return rc;
    if (cfg->encoder != PRODM_ENC_NEGABINARY && cfg->encoder != PRODM_ENC_GROUPED && cfg->encoder != PRODM_ENC_PERBIT)
        return fail(PRODM_EINVAL, "unknown encoder");
    // the per-bit encoder's error-collecting overload shifts 32-bit integers by
    // up to B-1 bits (PerBitBPEncoder.hpp:388-397); its drivers use the max collector
    if (cfg->encoder == PRODM_ENC_PERBIT && cfg->collector == PRODM_COLLECT_SQUARED)
        return fail(PRODM_EUNSUPPORTED, "the per-bit encoder is used with PRODM_COLLECT_MAX");
    if (cfg->basis != PRODM_BASIS_HIERARCHICAL && cfg->basis != PRODM_BASIS_ORTHOGONAL) return fail(PRODM_EINVAL, "unknown basis");
    if ((rc = check_bitplanes(cfg->dtype, cfg->encoder, cfg->num_bitplanes))) return rc;
    if (cfg->ndims < 1 || cfg->ndims > 3) return fail(PRODM_EINVAL, "ndims must be 1, 2 or 3");
    int ml = max_level(cfg->ndims, cfg->dims);
    if (cfg->target_level < 0 || cfg->target_level > ml)   // ComposedRefactor.hpp:79-83
        return fail(PRODM_EINVAL, "Target level is higher than " + std::to_string(ml));
    prodm_mdr* h = new prodm_mdr();
    h->cfg = *cfg;
    if ((rc = make_geom(cfg->ndims, cfg->dims, cfg->target_level, h->g))) { delete h; return rc; }
    h->B = cfg->num_bitplanes;
    h->es = esize(cfg->dtype);
    h->nb = cfg->encoder == PRODM_ENC_NEGABINARY;
    h->pb = cfg->encoder == PRODM_ENC_PERBIT;
    h->orth = cfg->basis == PRODM_BASIS_ORTHOGONAL;
    h->sq = cfg->collector == PRODM_COLLECT_SQUARED;
    if ((rc = mdr_alloc_all(h))) { delete h; return rc; }
    *out = h;
    return PRODM_OK;
}

static int mdr_lossless_sizes(prodm_mdr* h, cudaStream_t st);

int prodm_mdr_refactor(prodm_mdr* h, const void* field, void* stream) {
    if (!h || !field) return fail(PRODM_EINVAL, "prodm_mdr_refactor: NULL pointer");
    h->after_reconstruct = false;
    cudaStream_t st = (cudaStream_t)stream;
    if (h->from_files) h->ll_latter = -1;   // a loaded stage does not carry over to a new refactor
    h->from_files = false;
    h->hsz_valid = false;
    const int rc = h->cfg.dtype == PRODM_F64 ? mdr_refactor<double>(h, (const double*)field, st)
                                             : mdr_refactor<float>(h, (const float*)field, st);
    if (rc) return rc;
    h->refactored = true;
    return h->ll_latter >= 0 ? mdr_lossless_sizes(h, st) : PRODM_OK;
}

int prodm_mdr_level_info(prodm_mdr* h, uint32_t* hs, double* hb, double* he, void* stream) {
    if (!h) return fail(PRODM_EINVAL, "NULL handle");
    cudaStream_t st = (cudaStream_t)stream;
    const int L = h->g.L, B = h->B;
    if (hs) PRODM_CUDA(cudaMemcpyAsync(hs, h->sizes, (L + 1) * B * 4, cudaMemcpyDeviceToHost, st));
    std::vector<uint8_t> b((L + 1) * h->es);
    if (hb) PRODM_CUDA(cudaMemcpyAsync(b.data(), h->bounds, b.size(), cudaMemcpyDeviceToHost, st));
    if (he) PRODM_CUDA(cudaMemcpyAsync(he, h->sqerr, (L + 1) * (B + 1) * 8, cudaMemcpyDeviceToHost, st));
    PRODM_CUDA(cudaStreamSynchronize(st));
    if (hb)
        for (int l = 0; l <= L; l++)
            hb[l] = h->es == 8 ? ((double*)b.data())[l] : (double)((float*)b.data())[l];
    return PRODM_OK;
}

int prodm_mdr_metadata(prodm_mdr* h, uint8_t* buf, size_t cap, size_t* len, void* stream) {
    if (!h || !len) return fail(PRODM_EINVAL, "NULL pointer");
    const int L = h->g.L, B = h->B, nl = L + 1, nd = h->g.ndims;
    // ComposedRefactor.hpp:48-67 + extension: "SQER" u32 (B+1) doubles per level
    size_t need = 1 + 4 * nd + 1 + nl * h->es + nl * (4 + 4 * B) + nl + 4 * nl + 1 + 4 + 4 + nl * (B + 1) * 8 +
                  (h->ll_latter >= 0 ? 8 : 0);
    *len = need;
    if (!buf) return PRODM_OK;
    if (cap < need) return fail(PRODM_EINVAL, "metadata buffer too small");
    std::vector<uint32_t> sz(nl * B);
    std::vector<uint8_t> bd(nl * h->es);
    std::vector<double> er(nl * (B + 1));
    cudaStream_t st = (cudaStream_t)stream;
    PRODM_CUDA(cudaMemcpyAsync(sz.data(), h->sizes, sz.size() * 4, cudaMemcpyDeviceToHost, st));
    PRODM_CUDA(cudaMemcpyAsync(bd.data(), h->bounds, bd.size(), cudaMemcpyDeviceToHost, st));
    PRODM_CUDA(cudaMemcpyAsync(er.data(), h->sqerr, er.size() * 8, cudaMemcpyDeviceToHost, st));
    PRODM_CUDA(cudaStreamSynchronize(st));
    uint8_t* p = buf;
    *p++ = (uint8_t)nd;
    memcpy(p, h->g.dims, 4 * nd); p += 4 * nd;
    *p++ = (uint8_t)nl;
    memcpy(p, bd.data(), bd.size()); p += bd.size();
    for (int l = 0; l < nl; l++) {
        uint32_t c = B;
        memcpy(p, &c, 4); p += 4;
        memcpy(p, sz.data() + l * B, 4 * B); p += 4 * B;
    }
    for (int l = 0; l < nl; l++) *p++ = h->ll_latter >= 0 ? h->ll_stop[l] : 0;   // stopping indices
    for (int l = 0; l < nl; l++) { uint32_t one = 1; memcpy(p, &one, 4); p += 4; }   // level_num
    *p++ = (uint8_t)(h->nb ? 1 : 0);
    memcpy(p, "SQER", 4); p += 4;
    uint32_t cnt = (uint32_t)(B + 1);
    memcpy(p, &cnt, 4); p += 4;
    memcpy(p, er.data(), er.size() * 8); p += er.size() * 8;
    if (h->ll_latter >= 0) {   // the lossless stage's codec and latter index
        memcpy(p, "ZCB1", 4); p += 4;
        uint32_t lt = (uint32_t)h->ll_latter;
        memcpy(p, &lt, 4); p += 4;
    }
    return PRODM_OK;
}

// the level file with raw (uncompressed) streams; dsizes: the level's raw
// plane sizes on the device
// (hsizes: the same on the host when the caller has them, else NULL);
// dst_is_host == 2: pinned host memory, left to complete in stream order
static int export_raw_level(prodm_mdr* h, int level, void* dst, uint64_t cap, int dst_is_host, uint64_t* len,
                            const uint32_t* dsizes, cudaStream_t st, const uint32_t* hsizes = nullptr) {
    const int B = h->B;
    const bool async = dst_is_host == 2;
    std::vector<uint32_t> sz(B);
    if (hsizes) {
        std::memcpy(sz.data(), hsizes, B * 4);
    } else {
        PRODM_CUDA(cudaMemcpyAsync(sz.data(), dsizes, B * 4, cudaMemcpyDeviceToHost, st));
        PRODM_CUDA(cudaStreamSynchronize(st));
    }
    uint64_t total = 0;
    for (int p = 0; p < B; p++) total += sz[p];
    if (len) *len = total;
    if (!dst) return PRODM_OK;
    if (cap < total) return fail(PRODM_EINVAL, "export buffer too small");
    const uint8_t* src = h->streams + h->lvl_byte_off[level];
    if (h->nb) {   // padded plane rows -> the contiguous level-file layout
        const size_t row = (size_t)h->nblocks[level] * h->es;
        PRODM_CUDA(cudaMemcpy2DAsync(dst, row, src, (size_t)h->plane_cap[level] * h->es, row, B,
                                     dst_is_host ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice, st));
        if (!async) PRODM_CUDA(cudaStreamSynchronize(st));
        return PRODM_OK;
    }
    if (h->pb) {   // rows -> reference streams (8-byte aligned staging where dst is not)
        const bool direct = !dst_is_host && (uintptr_t)dst % 8 == 0;
        const uint64_t n = h->g.elems[level];
        const size_t scr = pb_pack_scratch_bytes(n, B);
        uint8_t* tmp;
        PRODM_CUDA(cudaMallocAsync((void**)&tmp, scr + (direct ? 0 : (total + 255) / 256 * 256), st));
        uint8_t* out = direct ? (uint8_t*)dst : tmp + scr;
        const uint32_t* rows = (const uint32_t*)src;
        int rc = launch_pb_pack(rows, h->plane_cap[level], n, B, dsizes, total,
                                out, tmp, st);
        if (!rc && !direct) {
            const cudaError_t e = cudaMemcpyAsync(dst, out, total,
                                                  dst_is_host ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice, st);
            if (e != cudaSuccess) rc = cuda_status(e, "export copy");
        }
        cudaFreeAsync(tmp, st);
        if (rc) return rc;
        if (!async) PRODM_CUDA(cudaStreamSynchronize(st));
        return PRODM_OK;
    }
    uint8_t* tmp = (uint8_t*)dst;
    if (dst_is_host) PRODM_CUDA(cudaMallocAsync((void**)&tmp, total, st));
    int rc = launch_gr_pack((const void* const*)(h->plane_ptrs + (uint64_t)level * B), dsizes, B,
                            h->nblocks[level], h->rbs + h->rb_off[level], (int)h->es, tmp, st);
    if (rc) return rc;
    if (dst_is_host) {
        PRODM_CUDA(cudaMemcpyAsync(dst, tmp, total, cudaMemcpyDeviceToHost, st));
        cudaFreeAsync(tmp, st);
    }
    if (!async) PRODM_CUDA(cudaStreamSynchronize(st));
    return PRODM_OK;
}

// lossless stage on: the encoders' (raw) sizes -> rsizes; per level the raw
// level file is built in scratch, each stream's ZCB size counted and the
// adaptive rule applied; the stored sizes -> sizes (the interpreter's cost
// model, as the reference's metadata carries them)
static int mdr_lossless_sizes(prodm_mdr* h, cudaStream_t st) {
    const int nl = h->g.L + 1, B = h->B;
    std::vector<uint32_t> raw(nl * B), stored(nl * B);
    if (h->nb) {   // fixed raw sizes (the refactor does not rewrite them)
        for (int l = 0; l < nl; l++)
            for (int p = 0; p < B; p++) raw[l * B + p] = (uint32_t)(h->nblocks[l] * h->es);
        PRODM_CUDA(cudaMemcpyAsync(h->rsizes, raw.data(), nl * B * 4, cudaMemcpyHostToDevice, st));
    } else {
        PRODM_CUDA(cudaMemcpyAsync(h->rsizes, h->sizes, nl * B * 4, cudaMemcpyDeviceToDevice, st));
        PRODM_CUDA(cudaMemcpyAsync(raw.data(), h->sizes, nl * B * 4, cudaMemcpyDeviceToHost, st));
    }
    PRODM_CUDA(cudaStreamSynchronize(st));
    h->ll_stop.assign(nl, 0);
    h->ll_flags.assign((size_t)nl * B, 0);
    uint64_t maxraw = 0;
    for (int l = 0; l < nl; l++) {
        uint64_t t = 0;
        for (int p = 0; p < B; p++) t += raw[l * B + p];
        maxraw = t > maxraw ? t : maxraw;
    }
    uint8_t* tmp;
    PRODM_CUDA(cudaMallocAsync((void**)&tmp, maxraw + 256, st));
    int rc = PRODM_OK;
    std::vector<uint32_t> comp(B);
    for (int l = 0; l < nl && !rc; l++) {
        rc = export_raw_level(h, l, tmp, maxraw, 0, nullptr, h->rsizes + (uint64_t)l * B, st);
        if (!rc) rc = ll_stream_sizes(tmp, raw.data() + l * B, B, comp.data(), st);
        if (rc) break;
        h->ll_stop[l] = (uint8_t)adaptive_stopping(raw.data() + l * B, comp.data(), B, h->ll_latter,
                                                    h->ll_flags.data() + (size_t)l * B);
        for (int p = 0; p < B; p++) stored[l * B + p] = h->ll_flags[(size_t)l * B + p] ? comp[p] : raw[l * B + p];
    }
    cudaFreeAsync(tmp, st);
    if (rc) return rc;
    PRODM_CUDA(cudaMemcpyAsync(h->sizes, stored.data(), nl * B * 4, cudaMemcpyHostToDevice, st));
    PRODM_CUDA(cudaStreamSynchronize(st));
    return PRODM_OK;
}

int prodm_mdr_export_level(prodm_mdr* h, int level, void* dst, uint64_t cap, int dst_is_host, uint64_t* len, void* stream) {
    if (!h) return fail(PRODM_EINVAL, "NULL handle");
    const int L = h->g.L, B = h->B;
    if (level < 0 || level > L) return fail(PRODM_EINVAL, "level out of range");
    cudaStream_t st = (cudaStream_t)stream;
    if (dst_is_host < 0 || dst_is_host > 2) return fail(PRODM_EINVAL, "dst_is_host must be 0, 1 or 2");
    if (h->ll_latter < 0) {
        // the plane sizes, on the host once per refactor: later exports need no
        // synchronisation before their copies
        if (!h->hsz_valid) {
            h->hsz.resize((size_t)(L + 1) * B);
            PRODM_CUDA(cudaMemcpyAsync(h->hsz.data(), h->sizes, (L + 1) * B * 4, cudaMemcpyDeviceToHost, st));
            PRODM_CUDA(cudaStreamSynchronize(st));
            h->hsz_valid = true;
        }
        return export_raw_level(h, level, dst, cap, dst_is_host, len, h->sizes + (uint64_t)level * B, st,
                                h->hsz.data() + (size_t)level * B);
    }
    // lossless stage: the raw level into scratch, then its stored streams
    std::vector<uint32_t> raw(B), stored(B);
    PRODM_CUDA(cudaMemcpyAsync(raw.data(), h->rsizes + (uint64_t)level * B, B * 4, cudaMemcpyDeviceToHost, st));
    PRODM_CUDA(cudaMemcpyAsync(stored.data(), h->sizes + (uint64_t)level * B, B * 4, cudaMemcpyDeviceToHost, st));
    PRODM_CUDA(cudaStreamSynchronize(st));
    uint64_t rtotal = 0, total = 0;
    for (int p = 0; p < B; p++) { rtotal += raw[p]; total += stored[p]; }
    if (len) *len = total;
    if (!dst) return PRODM_OK;
    if (cap < total) return fail(PRODM_EINVAL, "export buffer too small");
    uint8_t* tmp;
    const uint64_t rpad = (rtotal + 255) / 256 * 256;
    PRODM_CUDA(cudaMallocAsync((void**)&tmp, rpad + (dst_is_host ? total + 256 : 256), st));
    int rc = export_raw_level(h, level, tmp, rtotal, 0, nullptr, h->rsizes + (uint64_t)level * B, st);
    uint8_t* out = dst_is_host ? tmp + rpad : (uint8_t*)dst;
    std::vector<uint32_t> osz(B);
    int stop = 0;
    if (!rc)
        rc = ll_compress_level(tmp, raw.data(), B, h->ll_latter, out, total, osz.data(), &stop,
                               h->ll_flags.data() + (size_t)level * B, st);
    if (!rc && dst_is_host) {
        cudaError_t e = cudaMemcpyAsync(dst, out, total, cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) rc = cuda_status(e, "export copy");
    }
    cudaFreeAsync(tmp, st);
    return rc;
}

int prodm_mdr_export_level_range(prodm_mdr* h, int level, uint64_t offset, uint64_t bytes, void* dst,
                                 int dst_is_host, void* stream) {
    if (!h || (!dst && bytes)) return fail(PRODM_EINVAL, "NULL pointer");
    if (level < 0 || level > h->g.L) return fail(PRODM_EINVAL, "level out of range");
    if (dst_is_host < 0 || dst_is_host > 2) return fail(PRODM_EINVAL, "dst_is_host must be 0, 1 or 2");
    cudaStream_t st = (cudaStream_t)stream;
    uint64_t total = 0;
    int rc = prodm_mdr_export_level(h, level, nullptr, 0, 0, &total, stream);
    if (rc) return rc;
    if (offset > total || bytes > total - offset) return fail(PRODM_EINVAL, "byte range past the end of the level file");
    if (!bytes) return PRODM_OK;
    const cudaMemcpyKind kind = dst_is_host ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice;
    uint8_t* out = (uint8_t*)dst;
    if (h->nb && h->ll_latter < 0) {
        // fixed-size plane rows: the range is a tail of one row, whole rows, a head of one row
        const uint64_t row = h->nblocks[level] * h->es, pitch = (uint64_t)h->plane_cap[level] * h->es;
        const uint8_t* src = h->streams + h->lvl_byte_off[level];
        uint64_t a = offset;
        const uint64_t b = offset + bytes;
        if (a % row) {
            const uint64_t n = std::min(b, (a / row + 1) * row) - a;
            PRODM_CUDA(cudaMemcpyAsync(out, src + (a / row) * pitch + a % row, n, kind, st));
            out += n;
            a += n;
        }
        if (b - a >= row) {
            const uint64_t rows = (b - a) / row;
            PRODM_CUDA(cudaMemcpy2DAsync(out, row, src + (a / row) * pitch, pitch, row, rows, kind, st));
            out += rows * row;
            a += rows * row;
        }
        if (a < b) PRODM_CUDA(cudaMemcpyAsync(out, src + (a / row) * pitch, b - a, kind, st));
    } else {   // the whole file into device scratch, then the range
        uint8_t* tmp;
        PRODM_CUDA(cudaMallocAsync((void**)&tmp, total, st));
        uint64_t len = 0;
        rc = prodm_mdr_export_level(h, level, tmp, total, 0, &len, stream);
        if (!rc) {
            const cudaError_t e = cudaMemcpyAsync(out, tmp + offset, bytes, kind, st);
            if (e != cudaSuccess) rc = cuda_status(e, "export copy");
        }
        cudaFreeAsync(tmp, st);
        if (rc) return rc;
    }
    if (dst_is_host == 1) PRODM_CUDA(cudaStreamSynchronize(st));
    return PRODM_OK;
}

int prodm_mdr_set_lossless(prodm_mdr* h, int latter_index, void* stream) {
    if (!h) return fail(PRODM_EINVAL, "NULL handle");
    h->after_reconstruct = false;
    if (h->from_files) return fail(PRODM_EINVAL, "set_lossless: a handle fed from files takes the stage from its metadata");
    h->hsz_valid = false;
    cudaStream_t st = (cudaStream_t)stream;
    const int nl = h->g.L + 1, B = h->B;
    if (latter_index < 0) {   // off: the raw sizes back to the cost model
        if (h->ll_latter >= 0) PRODM_CUDA(cudaMemcpyAsync(h->sizes, h->rsizes, nl * B * 4, cudaMemcpyDeviceToDevice, st));
        h->ll_latter = -1;
        return PRODM_OK;
    }
    if (h->ll_latter >= 0) PRODM_CUDA(cudaMemcpyAsync(h->sizes, h->rsizes, nl * B * 4, cudaMemcpyDeviceToDevice, st));
    h->ll_latter = latter_index;
    return h->refactored ? mdr_lossless_sizes(h, st) : PRODM_OK;
}

int prodm_mdr_set_zstd_latter(prodm_mdr* h, int latter_index) {
    if (!h) return fail(PRODM_EINVAL, "NULL handle");
    if (latter_index < 0 || latter_index > 255) return fail(PRODM_EINVAL, "set_zstd_latter: latter index outside 0..255");
    h->zstd_latter = latter_index;
    return PRODM_OK;
}

int prodm_mdr_retrieve(prodm_mdr* h, double tol, int interp, int est, double s, void* out, void* stream) {
    if (!h || !out) return fail(PRODM_EINVAL, "prodm_mdr_retrieve: NULL pointer");
    if (interp < 0 || interp > 2 || est < 0 || est > 3) return fail(PRODM_EINVAL, "unknown interpreter or estimator");
    cudaStream_t st = (cudaStream_t)stream;
    if (h->cfg.dtype == PRODM_F64) return mdr_retrieve<double>(h, tol, interp, est, s, (double*)out, st);
    return mdr_retrieve<float>(h, tol, interp, est, s, (float*)out, st);
}

int prodm_mdr_interpret(prodm_mdr* h, double tol, int interp, int est, double s, void* stream) {
    if (!h) return fail(PRODM_EINVAL, "NULL handle");
    if (interp < 0 || interp > 2 || est < 0 || est > 3) return fail(PRODM_EINVAL, "unknown interpreter or estimator");
    cudaStream_t st = (cudaStream_t)stream;
    if (h->cfg.dtype == PRODM_F64) return mdr_interpret<double>(h, tol, interp, est, s, st);
    return mdr_interpret<float>(h, tol, interp, est, s, st);
}

int prodm_mdr_reconstruct(prodm_mdr* h, void* out, void* stream) {
    if (!h || !out) return fail(PRODM_EINVAL, "NULL pointer");
    cudaStream_t st = (cudaStream_t)stream;
    if (h->cfg.dtype == PRODM_F64) return mdr_reconstruct<double>(h, (double*)out, st);
    return mdr_reconstruct<float>(h, (float*)out, st);
}

int prodm_mdr_load_metadata(prodm_mdr* h, const uint8_t* buf, size_t len, void* stream) {
    if (!h || !buf) return fail(PRODM_EINVAL, "NULL pointer");
    h->after_reconstruct = false;
    cudaStream_t st = (cudaStream_t)stream;
    if (h->cfg.dtype == PRODM_F64) return mdr_load_metadata<double>(h, buf, len, st);
    return mdr_load_metadata<float>(h, buf, len, st);
}

int prodm_mdr_load_level(prodm_mdr* h, int level, const void* src, uint64_t off, uint64_t bytes, int host, void* stream) {
    if (!h || (!src && bytes)) return fail(PRODM_EINVAL, "NULL pointer");
    h->after_reconstruct = false;
    if (level < 0 || level > h->g.L) return fail(PRODM_EINVAL, "level out of range");
    if (h->from_files && h->ll_latter >= 0) return mdr_ll_load(h, level, src, off, bytes, host, (cudaStream_t)stream);
    return mdr_load_level(h, level, src, off, bytes, host, (cudaStream_t)stream);
}

int prodm_mdr_load_level_file(prodm_mdr* h, int level, const char* path, uint64_t file_offset, uint64_t level_offset,
                              uint64_t bytes, void* stream) {
    if (!h || !path) return fail(PRODM_EINVAL, "NULL pointer");
    h->after_reconstruct = false;
    if (level < 0 || level > h->g.L) return fail(PRODM_EINVAL, "level out of range");
    if (!h->from_files) return fail(PRODM_EINVAL, "load_level_file: load the metadata first");
    cudaStream_t st = (cudaStream_t)stream;
    auto sink = [&](const void* src, uint64_t at, uint64_t n, int host) -> int {
        return h->ll_latter >= 0 ? mdr_ll_load(h, level, src, level_offset + at, n, host, st)
                                 : mdr_load_level(h, level, src, level_offset + at, n, host, st);
    };
    return read_file_range(h->fstage, path, file_offset, bytes, sink, st, nullptr);
}

int prodm_mdr_write_level_file(prodm_mdr* h, int level, const char* path, void* stream) {
    if (!h || !path) return fail(PRODM_EINVAL, "NULL pointer");
    uint64_t len = 0;
    int rc = prodm_mdr_export_level(h, level, nullptr, 0, 1, &len, stream);
    if (rc) return rc;
    std::vector<uint8_t> buf(len);
    if ((rc = prodm_mdr_export_level(h, level, buf.data(), len, 1, &len, stream))) return rc;
    FILE* f = std::fopen(path, "wb");
    if (!f) return fail(PRODM_EINVAL, std::string("cannot write ") + path);
    const size_t w = len ? std::fwrite(buf.data(), 1, len, f) : 0;
    const int c = std::fclose(f);
    if (w != len || c != 0) return fail(PRODM_EINVAL, std::string("short write to ") + path);
    return PRODM_OK;
}

int prodm_mdr_file_read_mode(prodm_mdr* h, int* mode) {
    if (!h || !mode) return fail(PRODM_EINVAL, "NULL pointer");
    *mode = h->fstage ? file_staging_mode(h->fstage) : -1;
    return PRODM_OK;
}

int prodm_mdr_retrieve_planes(prodm_mdr* h, const uint8_t* hidx, void* out, void* stream) {
    if (!h || !out || !hidx) return fail(PRODM_EINVAL, "prodm_mdr_retrieve_planes: NULL pointer");
    const int L = h->g.L;
    for (int l = 0; l <= L; l++)
        if (hidx[l] > h->B) return fail(PRODM_EINVAL, "plane count above num_bitplanes");
    cudaStream_t st = (cudaStream_t)stream;
    PRODM_CUDA(cudaMemcpyAsync(h->index, hidx, L + 1, cudaMemcpyHostToDevice, st));
    PRODM_CUDA(cudaStreamSynchronize(st));
    if (h->cfg.dtype == PRODM_F64) return mdr_reconstruct<double>(h, (double*)out, st);
    return mdr_reconstruct<float>(h, (float*)out, st);
}

// The plane counts and the retrieval status are read back through mapped
// host memory written by a one-block kernel: a small copy on a copy engine
// would wait behind any large device-to-host copy already queued there (the
// previous reconstruction on its way to the host, for instance).
static __global__ void k_read_index(const uint8_t* __restrict__ idx, int n, const int* __restrict__ status,
                                    uint8_t* __restrict__ map) {
    const int t = threadIdx.x;
    if (t < n) map[t] = idx[t];
    if (t == 0) *reinterpret_cast<volatile int*>(map + 64) = *status;
    __threadfence_system();
}

static int read_index(prodm_mdr* h, uint8_t* hidx, cudaStream_t st, int* code) {
    const int n = hidx ? h->g.L + 1 : 0;
    k_read_index<<<1, 64, 0, st>>>(h->index, n, h->kstatus, h->dmap);
    PRODM_CHECK_LAUNCH("k_read_index");
    PRODM_CUDA(cudaStreamSynchronize(st));
    if (n) std::memcpy(hidx, h->hmap, n);
    *code = *reinterpret_cast<volatile int*>(h->hmap + 64);
    return PRODM_OK;
}

// the retrieval kernels' bounded waits: a nonzero code is reported once and cleared
static int report_kstatus(prodm_mdr* h, int code, cudaStream_t st) {
    if (!code) return PRODM_OK;
    PRODM_CUDA(cudaMemsetAsync(h->kstatus, 0, 4, st));
    PRODM_CUDA(cudaStreamSynchronize(st));
    if (code == PRODM_ETIMEOUT) return fail(PRODM_ETIMEOUT, "a retrieval kernel's bounded wait for its plane tiles gave up");
    return fail(code, "a retrieval kernel found its shared memory misaligned for TMA");
}

int prodm_mdr_get_index(prodm_mdr* h, uint8_t* hidx, void* stream) {
    if (!h || !hidx) return fail(PRODM_EINVAL, "NULL pointer");
    cudaStream_t st = (cudaStream_t)stream;
    int code = 0, rc;
    if ((rc = read_index(h, hidx, st, &code))) return rc;
    return report_kstatus(h, code, st);
}

int prodm_mdr_status(prodm_mdr* h, void* stream) {
    if (!h) return fail(PRODM_EINVAL, "NULL handle");
    cudaStream_t st = (cudaStream_t)stream;
    int code = 0, rc;
    if ((rc = read_index(h, nullptr, st, &code))) return rc;
    return report_kstatus(h, code, st);
}

int prodm_debug_tile_wait(int extra_tx_bytes, long long wait_cycles) {
    if (extra_tx_bytes < 0 || extra_tx_bytes > (1 << 16)) return fail(PRODM_EINVAL, "extra_tx_bytes out of range");
    prodm::fused_tma_test_hook(extra_tx_bytes, wait_cycles);
    return PRODM_OK;
}

int prodm_mdr_reset_retrieval(prodm_mdr* h, void* stream) {
    if (!h) return fail(PRODM_EINVAL, "NULL handle");
    h->after_reconstruct = false;
    PRODM_CUDA(cudaMemsetAsync(h->index, 0, h->g.L + 1, (cudaStream_t)stream));
    return PRODM_OK;
}

int prodm_mdr_coefficients(prodm_mdr* h, void* dst, void* stream) {
    if (!h || !dst) return fail(PRODM_EINVAL, "NULL pointer");
    cudaStream_t st = (cudaStream_t)stream;
    PRODM_CUDA(cudaMemcpyAsync(dst, h->coef, h->g.total * h->es, cudaMemcpyDeviceToDevice, st));
    return PRODM_OK;
}

int prodm_mdr_set_timing(prodm_mdr* h, int enable) {
    if (!h) return fail(PRODM_EINVAL, "NULL handle");
    int rc = h->collect();
    if (rc) return rc;
    h->timing = enable != 0;
    for (int i = 0; i < 5 * 17; i++) { h->stage_ms[i] = 0; h->stage_n[i] = 0; }
    return PRODM_OK;
}

int prodm_mdr_stage_times(prodm_mdr* h, double* ms, uint32_t* counts) {
    if (!h || !ms || !counts) return fail(PRODM_EINVAL, "NULL pointer");
    int rc = h->collect();
    if (rc) return rc;
    for (int i = 0; i < 5 * 17; i++) { ms[i] = h->stage_ms[i]; counts[i] = h->stage_n[i]; }
    return PRODM_OK;
}

int prodm_kernel_launch_count(uint64_t* out) {
    if (!out) return fail(PRODM_EINVAL, "NULL pointer");
    *out = g_launches.load();
    return PRODM_OK;
}

int prodm_mdr_destroy(prodm_mdr* h) {
    delete h;
    return PRODM_OK;
}

}  // extern "C"
