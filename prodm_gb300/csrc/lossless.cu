// Lossless stage on the device (sm_103a): the ZCB codec (zero-compacted
// bytes; this project's format, not zstd) and AdaptiveLevelCompressor's
// stopping rule (AdaptiveLevelCompressor.hpp:13-40).
//
// A stream compresses as 4096-byte chunks of 32-bit words (the last word
// zero-padded), each independent of the others:
//   u64 raw length | u32 chunk count C | u32 end offset of each chunk's data
//   (relative to the end of this table) | chunk data
// chunk data: 32 u32 word masks (bit k of mask m: word 32m+k nonzero), a
// 4-bit byte mask per nonzero word (8 per u32, in word order, padded to a
// u32), the nonzero bytes in order (padded to 4 bytes). The raw length comes
// first as in the reference's zstd wrapper (ZSTD.hpp:9-20). One warp per
// chunk in all three passes: count (sizes, for the stopping rule and the
// retrieval cost model), write, read.
#include <cstring>
#include <vector>

#include "common.cuh"
#include "kernels.cuh"

namespace prodm {

namespace {

constexpr unsigned FULL = 0xffffffffu;
constexpr int ZW = 8;   // warps per CTA

__device__ __forceinline__ int zseg(const ZStream* s, int ns, uint64_t g) { return find_seg(s, ns, g, &ZStream::chunk0); }

// word w of chunk c (4 bytes, zero beyond the stream's end)
__device__ __forceinline__ uint32_t zword(const uint8_t* __restrict__ src, uint64_t len, uint64_t b) {
    if (b + 4 <= len && ((uintptr_t)(src + b) & 3) == 0) return __ldcs((const uint32_t*)(src + b));
    uint32_t w = 0;
    for (int k = 0; k < 4; k++)
        if (b + k < len) w |= (uint32_t)src[b + k] << (8 * k);
    return w;
}

__device__ __forceinline__ uint32_t nib_of(uint32_t w) {
    return (w & 0xffu ? 1u : 0u) | (w & 0xff00u ? 2u : 0u) | (w & 0xff0000u ? 4u : 0u) | (w & 0xff000000u ? 8u : 0u);
}

__device__ __forceinline__ uint32_t chunk_bytes(uint32_t nzw, uint32_t nzb) {
    return 128 + 4 * ((nzw + 7) / 8) + 4 * ((nzb + 3) / 4);
}

__global__ void __launch_bounds__(32 * ZW) k_zcb_count(const ZStream* __restrict__ ss, int ns, uint64_t total,
                                                       uint32_t* __restrict__ csize) {
    const int lane = threadIdx.x & 31;
    for (uint64_t g = (uint64_t)blockIdx.x * ZW + (threadIdx.x >> 5); g < total; g += (uint64_t)gridDim.x * ZW) {
        const ZStream s = ss[zseg(ss, ns, g)];
        const uint64_t base = (g - s.chunk0) * 4096;
        uint32_t nzw = 0, nzb = 0;
#pragma unroll 4
        for (int i = 0; i < 32; i++) {
            const uint32_t w = zword(s.src, s.len, base + 4 * (32 * i + lane));
            nzw += __popc(__ballot_sync(FULL, w != 0));
            nzb += __reduce_add_sync(FULL, __popc(nib_of(w)));
        }
        if (lane == 0) csize[g] = chunk_bytes(nzw, nzb);
    }
}

// per stream: chunk data offsets (exclusive scan) and the compressed size
__global__ void k_zcb_scan(const ZStream* __restrict__ ss, const uint32_t* __restrict__ csize,
                           uint32_t* __restrict__ coff, uint32_t* __restrict__ out_size) {
    const ZStream s = ss[blockIdx.x];
    const int lane = threadIdx.x;
    const uint64_t nch = (s.len + 4095) / 4096;
    uint32_t run = 0;
    for (uint64_t c0 = 0; c0 < nch; c0 += 32) {
        const uint64_t c = c0 + lane;
        const uint32_t v = c < nch ? csize[s.chunk0 + c] : 0u;
        uint32_t inc = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t t = __shfl_up_sync(FULL, inc, o);
            if (lane >= o) inc += t;
        }
        if (c < nch) coff[s.chunk0 + c] = run + inc - v;
        run += __shfl_sync(FULL, inc, 31);
    }
    if (lane == 0) out_size[blockIdx.x] = (uint32_t)(12 + 4 * nch + run);
}

// dst of each stream: 4-byte aligned, its compressed size long
__global__ void __launch_bounds__(32 * ZW) k_zcb_write(const ZStream* __restrict__ ss, int ns, uint64_t total,
                                                       const uint32_t* __restrict__ csize,
                                                       const uint32_t* __restrict__ coff) {
    __shared__ uint32_t nibs[ZW][128];
    __shared__ uint32_t bytes[ZW][1024];
    const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
    const uint32_t lt = (1u << lane) - 1u;
    uint8_t* bb = (uint8_t*)bytes[wp];
    for (uint64_t g = (uint64_t)blockIdx.x * ZW + wp; g < total; g += (uint64_t)gridDim.x * ZW) {
        const ZStream s = ss[zseg(ss, ns, g)];
        const uint64_t c = g - s.chunk0, nch = (s.len + 4095) / 4096;
        const uint64_t base = c * 4096;
        uint32_t* out = (uint32_t*)s.dst;
        if (c == 0 && lane == 0) {
            out[0] = (uint32_t)s.len;
            out[1] = (uint32_t)(s.len >> 32);
            out[2] = (uint32_t)nch;
        }
        for (int k = lane; k < 128; k += 32) nibs[wp][k] = 0;
        __syncwarp();
        uint32_t nzw = 0, nzb = 0, mymask = 0;
        for (int i = 0; i < 32; i++) {
            const uint32_t w = zword(s.src, s.len, base + 4 * (32 * i + lane));
            const uint32_t m = __ballot_sync(FULL, w != 0);
            if (lane == i) mymask = m;
            const uint32_t nb = nib_of(w), cnt = __popc(nb);
            uint32_t inc = cnt;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t t = __shfl_up_sync(FULL, inc, o);
                if (lane >= o) inc += t;
            }
            if (w) {
                const uint32_t ord = nzw + __popc(m & lt);
                atomicOr(&nibs[wp][ord >> 3], nb << (4 * (ord & 7)));
                uint32_t at = nzb + inc - cnt;
                for (int k = 0; k < 4; k++)
                    if ((nb >> k) & 1u) bb[at++] = (uint8_t)(w >> (8 * k));
            }
            nzw += __popc(m);
            nzb += __shfl_sync(FULL, inc, 31);
        }
        if (lane == 0)
            for (uint32_t k = nzb; k & 3; k++) bb[k] = 0;
        __syncwarp();
        uint32_t* d = out + 3 + nch + coff[g] / 4;
        d[lane] = mymask;
        const uint32_t nn = (nzw + 7) / 8, nbw = (nzb + 3) / 4;
        for (uint32_t k = lane; k < nn; k += 32) d[32 + k] = nibs[wp][k];
        for (uint32_t k = lane; k < nbw; k += 32) d[32 + nn + k] = bytes[wp][k];
        if (lane == 0) out[3 + c] = coff[g] + csize[g];
        __syncwarp();
    }
}

// src of each stream: its compressed bytes, 4-byte aligned, `clen` long
// (headers checked on the host); dst: the raw bytes. A chunk whose offsets
// or counts do not fit its data records PRODM_ECORRUPT and is skipped.
__global__ void __launch_bounds__(32 * ZW) k_zcb_read(const ZStream* __restrict__ ss, int ns, uint64_t total,
                                                      int* __restrict__ status) {
    const int lane = threadIdx.x & 31;
    const uint32_t lt = (1u << lane) - 1u;
    for (uint64_t g = (uint64_t)blockIdx.x * ZW + (threadIdx.x >> 5); g < total; g += (uint64_t)gridDim.x * ZW) {
        const ZStream s = ss[zseg(ss, ns, g)];
        const uint64_t c = g - s.chunk0, nch = (s.len + 4095) / 4096;
        const uint32_t* in = (const uint32_t*)s.src;
        const uint64_t dlen = s.clen - 12 - 4 * nch;          // data area bytes
        const uint32_t start = c ? in[3 + c - 1] : 0u, end = in[3 + c];
        if (end < start + 128 || end > dlen || (start & 3) || (end & 3)) {
            if (lane == 0) atomicCAS(status, 0, PRODM_ECORRUPT);
            continue;
        }
        const uint32_t* d = in + 3 + nch + start / 4;
        const uint32_t clen = end - start;
        const uint32_t mymask = d[lane];
        const uint32_t nzw_all = __reduce_add_sync(FULL, __popc(mymask));
        const uint32_t nn = (nzw_all + 7) / 8;
        if (128 + 4 * nn > clen) {
            if (lane == 0) atomicCAS(status, 0, PRODM_ECORRUPT);
            continue;
        }
        const uint32_t* nib = d + 32;
        const uint8_t* by = (const uint8_t*)(d + 32 + nn);
        const uint32_t blen = clen - 128 - 4 * nn;
        uint32_t nzw = 0, nzb = 0;
        bool bad = false;
        const uint64_t base = c * 4096;
        for (int i = 0; i < 32; i++) {
            const uint32_t m = __shfl_sync(FULL, mymask, i);
            uint32_t nb = 0;
            if ((m >> lane) & 1u) {
                const uint32_t ord = nzw + __popc(m & lt);
                nb = (nib[ord >> 3] >> (4 * (ord & 7))) & 15u;
            }
            const uint32_t cnt = __popc(nb);
            uint32_t inc = cnt;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t t = __shfl_up_sync(FULL, inc, o);
                if (lane >= o) inc += t;
            }
            uint32_t at = nzb + inc - cnt, w = 0;
            for (int k = 0; k < 4; k++)
                if ((nb >> k) & 1u) {
                    if (at < blen) w |= (uint32_t)by[at] << (8 * k);
                    else bad = true;
                    at++;
                }
            const uint64_t b = base + 4 * (32 * i + lane);
            if (b + 4 <= s.len && ((uintptr_t)(s.dst + b) & 3) == 0) {
                *(uint32_t*)(s.dst + b) = w;
            } else {
                for (int k = 0; k < 4; k++)
                    if (b + k < s.len) s.dst[b + k] = (uint8_t)(w >> (8 * k));
            }
            nzw += __popc(m);
            nzb += __shfl_sync(FULL, inc, 31);
        }
        if (__any_sync(FULL, bad) && lane == 0) atomicCAS(status, 0, PRODM_ECORRUPT);
    }
}

unsigned zgrid(uint64_t chunks) {
    uint64_t g = (chunks + ZW - 1) / ZW;
    const uint64_t cap = (uint64_t)device_sms() * 8;
    return (unsigned)(g < 1 ? 1 : (g > cap ? cap : g));
}

}  // namespace

uint64_t zcb_bound(uint64_t len) {
    const uint64_t nch = (len + 4095) / 4096;
    return 12 + 4 * nch + nch * (128 + 512) + 4 * ((len + 3) / 4);
}

int launch_zcb_count(const ZStream* d_ss, int ns, uint64_t total_chunks, uint32_t* csize, uint32_t* coff,
                     uint32_t* out_sizes, cudaStream_t st) {
    if (total_chunks) {
        k_zcb_count<<<zgrid(total_chunks), 32 * ZW, 0, st>>>(d_ss, ns, total_chunks, csize);
        PRODM_CHECK_LAUNCH("k_zcb_count");
    }
    k_zcb_scan<<<ns, 32, 0, st>>>(d_ss, csize, coff, out_sizes);
    PRODM_CHECK_LAUNCH("k_zcb_scan");
    return PRODM_OK;
}

int launch_zcb_write(const ZStream* d_ss, int ns, uint64_t total_chunks, const uint32_t* csize, const uint32_t* coff,
                     cudaStream_t st) {
    if (!total_chunks) return PRODM_OK;
    k_zcb_write<<<zgrid(total_chunks), 32 * ZW, 0, st>>>(d_ss, ns, total_chunks, csize, coff);
    PRODM_CHECK_LAUNCH("k_zcb_write");
    return PRODM_OK;
}

int launch_zcb_read(const ZStream* d_ss, int ns, uint64_t total_chunks, int* status, cudaStream_t st) {
    if (!total_chunks) return PRODM_OK;
    k_zcb_read<<<zgrid(total_chunks), 32 * ZW, 0, st>>>(d_ss, ns, total_chunks, status);
    PRODM_CHECK_LAUNCH("k_zcb_read");
    return PRODM_OK;
}

// AdaptiveLevelCompressor::compress_level's rule on the given sizes
int adaptive_stopping(const uint32_t* raw, const uint32_t* comp, int B, int latter, uint8_t* compressed) {
    int stopping = B;
    for (int p = 0; p < B; p++) compressed[p] = 0;
    for (int i = 0; i < B; i++) {
        const float ratio = (float)(raw[i] * 1.0 / comp[i]);
        compressed[i] = 1;
        if (i && ratio < 1.05) {
            stopping = i;
            break;
        }
    }
    const int start = stopping < latter ? latter : stopping + 1;
    for (int i = start; i < B; i++) compressed[i] = 1;
    return stopping;
}

}  // namespace prodm

// ---------------------------------------------------------------------------
// host orchestration
// ---------------------------------------------------------------------------
namespace prodm {

namespace {
uint64_t align256(uint64_t x) { return (x + 255) / 256 * 256; }

// device descriptors + per-chunk scratch for `ss`; returns total chunks
struct ZJob {
    ZStream* d_ss = nullptr;
    uint32_t* csize = nullptr;
    uint32_t* coff = nullptr;
    uint32_t* outsz = nullptr;
    int* status = nullptr;
    uint8_t* base = nullptr;
    uint64_t chunks = 0;
    cudaStream_t st = nullptr;
    int setup(std::vector<ZStream>& ss, uint64_t extra, uint8_t** extra_out, cudaStream_t s) {
        st = s;
        chunks = 0;
        for (auto& z : ss) {
            z.chunk0 = chunks;
            chunks += (z.len + 4095) / 4096;
        }
        const uint64_t a = align256(ss.size() * sizeof(ZStream)), b = align256(chunks * 4 + 4),
                       c = align256(ss.size() * 4 + 4);
        PRODM_CUDA(cudaMallocAsync((void**)&base, a + 2 * b + c + 256 + extra, st));
        d_ss = (ZStream*)base;
        csize = (uint32_t*)(base + a);
        coff = (uint32_t*)(base + a + b);
        outsz = (uint32_t*)(base + a + 2 * b);
        status = (int*)(base + a + 2 * b + c);
        if (extra_out) *extra_out = base + a + 2 * b + c + 256;
        PRODM_CUDA(cudaMemcpyAsync(d_ss, ss.data(), ss.size() * sizeof(ZStream), cudaMemcpyHostToDevice, st));
        PRODM_CUDA(cudaMemsetAsync(status, 0, 4, st));
        return PRODM_OK;
    }
    ~ZJob() {
        if (base) cudaFreeAsync(base, st);
    }
};
}  // namespace

int ll_stream_sizes(const uint8_t* d_raw, const uint32_t* h_sizes, int B, uint32_t* h_comp, cudaStream_t st) {
    std::vector<ZStream> ss(B);
    uint64_t o = 0;
    for (int p = 0; p < B; p++) {
        ss[p] = ZStream{d_raw + o, nullptr, h_sizes[p], 0, 0};
        o += h_sizes[p];
    }
    ZJob j;
    int rc = j.setup(ss, 0, nullptr, st);
    if (rc) return rc;
    if ((rc = launch_zcb_count(j.d_ss, B, j.chunks, j.csize, j.coff, j.outsz, st))) return rc;
    PRODM_CUDA(cudaMemcpyAsync(h_comp, j.outsz, B * 4, cudaMemcpyDeviceToHost, st));
    PRODM_CUDA(cudaStreamSynchronize(st));
    return PRODM_OK;
}

int ll_compress_level(const uint8_t* d_raw, const uint32_t* h_sizes, int B, int latter, uint8_t* d_out, uint64_t cap,
                      uint32_t* h_out_sizes, int* h_stop, const uint8_t* h_flags, cudaStream_t st) {
    std::vector<ZStream> ss(B);
    std::vector<uint64_t> doff(B);
    uint64_t o = 0, scr = 0;
    for (int p = 0; p < B; p++) {
        ss[p] = ZStream{d_raw + o, nullptr, h_sizes[p], 0, 0};
        doff[p] = scr;
        scr += align256(zcb_bound(h_sizes[p]));
        o += h_sizes[p];
    }
    ZJob j;
    uint8_t* area = nullptr;
    int rc = j.setup(ss, scr, &area, st);
    if (rc) return rc;
    for (int p = 0; p < B; p++) ss[p].dst = area + doff[p];
    PRODM_CUDA(cudaMemcpyAsync(j.d_ss, ss.data(), ss.size() * sizeof(ZStream), cudaMemcpyHostToDevice, st));
    if ((rc = launch_zcb_count(j.d_ss, B, j.chunks, j.csize, j.coff, j.outsz, st))) return rc;
    std::vector<uint32_t> comp(B);
    PRODM_CUDA(cudaMemcpyAsync(comp.data(), j.outsz, B * 4, cudaMemcpyDeviceToHost, st));
    PRODM_CUDA(cudaStreamSynchronize(st));
    std::vector<uint8_t> flags(B);
    const int stop = adaptive_stopping(h_sizes, comp.data(), B, latter, flags.data());
    if (h_flags)
        for (int p = 0; p < B; p++) flags[p] = h_flags[p];
    uint64_t total = 0;
    for (int p = 0; p < B; p++) total += flags[p] ? comp[p] : h_sizes[p];
    if (total > cap) return fail(PRODM_EINVAL, "lossless: output capacity below the level's stored size");
    if ((rc = launch_zcb_write(j.d_ss, B, j.chunks, j.csize, j.coff, st))) return rc;
    o = 0;
    uint64_t r = 0;
    for (int p = 0; p < B; p++) {
        const uint64_t n = flags[p] ? comp[p] : h_sizes[p];
        if (n) PRODM_CUDA(cudaMemcpyAsync(d_out + o, flags[p] ? area + doff[p] : d_raw + r, n, cudaMemcpyDeviceToDevice, st));
        h_out_sizes[p] = (uint32_t)n;
        o += n;
        r += h_sizes[p];
    }
    if (h_stop) *h_stop = stop;
    PRODM_CUDA(cudaStreamSynchronize(st));
    return PRODM_OK;
}

int ll_decompress_planes(const uint8_t* d_in, const uint32_t* h_sizes, const uint8_t* h_flags, int num, uint8_t* d_out,
                         uint64_t cap, uint32_t* h_raw_sizes, cudaStream_t st) {
    // compressed streams -> 4-byte aligned staging; their headers to the host
    std::vector<uint64_t> soff(num), stage(num);
    uint64_t o = 0, scr = 0;
    for (int i = 0; i < num; i++) {
        soff[i] = o;
        o += h_sizes[i];
        stage[i] = scr;
        if (h_flags[i]) {
            if (h_sizes[i] < 12) return fail(PRODM_ECORRUPT, "lossless: compressed stream shorter than its header");
            scr += align256(h_sizes[i]);
        }
    }
    uint8_t* area = nullptr;
    if (scr) PRODM_CUDA(cudaMallocAsync((void**)&area, scr, st));
    struct Guard {
        uint8_t* p;
        cudaStream_t s;
        ~Guard() { if (p) cudaFreeAsync(p, s); }
    } guard{area, st};
    std::vector<uint8_t> hdr(12 * (size_t)num, 0);
    for (int i = 0; i < num; i++)
        if (h_flags[i]) {
            PRODM_CUDA(cudaMemcpyAsync(area + stage[i], d_in + soff[i], h_sizes[i], cudaMemcpyDeviceToDevice, st));
            PRODM_CUDA(cudaMemcpyAsync(hdr.data() + 12 * i, d_in + soff[i], 12, cudaMemcpyDeviceToHost, st));
        }
    PRODM_CUDA(cudaStreamSynchronize(st));
    std::vector<ZStream> ss;
    uint64_t r = 0;
    for (int i = 0; i < num; i++) {
        uint64_t len = h_sizes[i];
        if (h_flags[i]) {
            uint32_t nch;
            std::memcpy(&len, hdr.data() + 12 * i, 8);
            std::memcpy(&nch, hdr.data() + 12 * i + 8, 4);
            if (nch != (len + 4095) / 4096 || h_sizes[i] < 12 + 4 * (uint64_t)nch || len > 0xffffffffull)
                return fail(PRODM_ECORRUPT, "lossless: malformed compressed stream header");
        }
        if (r + len > cap) return fail(PRODM_EINVAL, "lossless: output capacity below the raw size");
        if (h_flags[i]) ss.push_back(ZStream{area + stage[i], d_out + r, len, h_sizes[i], 0});
        else if (len) PRODM_CUDA(cudaMemcpyAsync(d_out + r, d_in + soff[i], len, cudaMemcpyDeviceToDevice, st));
        h_raw_sizes[i] = (uint32_t)len;
        r += len;
    }
    if (ss.empty()) return PRODM_OK;
    ZJob j;
    int rc = j.setup(ss, 0, nullptr, st);
    if (rc) return rc;
    if ((rc = launch_zcb_read(j.d_ss, (int)ss.size(), j.chunks, j.status, st))) return rc;
    int hstat = 0;
    PRODM_CUDA(cudaMemcpyAsync(&hstat, j.status, 4, cudaMemcpyDeviceToHost, st));
    PRODM_CUDA(cudaStreamSynchronize(st));
    if (hstat) return fail(PRODM_ECORRUPT, "lossless: malformed compressed chunk");
    return PRODM_OK;
}

}  // namespace prodm

using namespace prodm;

extern "C" {

int prodm_lossless_compress_bound(const uint32_t* h_sizes, int num_bitplanes, uint64_t* out) {
    if (!h_sizes || !out || num_bitplanes < 1 || num_bitplanes > 64) return fail(PRODM_EINVAL, "bad arguments");
    uint64_t t = 0;
    for (int p = 0; p < num_bitplanes; p++) t += zcb_bound(h_sizes[p]) > h_sizes[p] ? zcb_bound(h_sizes[p]) : h_sizes[p];
    *out = t;
    return PRODM_OK;
}

int prodm_lossless_compress_level(const void* d_blob, const uint32_t* h_sizes, int num_bitplanes, int latter_index,
                                  void* d_out, uint64_t capacity, uint32_t* h_out_sizes, int* h_stopping_index,
                                  void* stream) {
    if (!d_blob || !h_sizes || !d_out || !h_out_sizes || !h_stopping_index || num_bitplanes < 1 || num_bitplanes > 64 ||
        latter_index < 0)
        return fail(PRODM_EINVAL, "prodm_lossless_compress_level: bad arguments");
    return ll_compress_level((const uint8_t*)d_blob, h_sizes, num_bitplanes, latter_index, (uint8_t*)d_out, capacity,
                             h_out_sizes, h_stopping_index, nullptr, (cudaStream_t)stream);
}

int prodm_lossless_decompress_level(const void* d_blob, const uint32_t* h_sizes, int starting_bitplane,
                                    int num_bitplanes, int stopping_index, int latter_index, void* d_out,
                                    uint64_t capacity, uint32_t* h_raw_sizes, void* stream) {
    if ((num_bitplanes > 0 && (!d_blob || !h_sizes || !d_out || !h_raw_sizes)) || starting_bitplane < 0 ||
        num_bitplanes < 0 || starting_bitplane + num_bitplanes > 64)
        return fail(PRODM_EINVAL, "prodm_lossless_decompress_level: bad arguments");
    std::vector<uint8_t> flags(num_bitplanes);
    for (int i = 0; i < num_bitplanes; i++) {   // AdaptiveLevelCompressor.hpp:43-52
        const int p = starting_bitplane + i;
        flags[i] = (p <= stopping_index || p >= latter_index) ? 1 : 0;
    }
    return ll_decompress_planes((const uint8_t*)d_blob, h_sizes, flags.data(), num_bitplanes, (uint8_t*)d_out,
                                capacity, h_raw_sizes, (cudaStream_t)stream);
}

}  // extern "C"
