// Negabinary fp32 codec bodies (bit transposes, chunk encode / decode),
// shared by the single-level kernels and the multi-field batched kernels.
#pragma once
#include "common.cuh"

namespace prodm {

// ---------------------------------------------------------------------------
// 32 x 32 bit transpose across a warp: lane e holds row e on entry; on exit
// lane k holds the word whose bit e is bit k of row e. Five exchange stages
// with the lane l ^ j: the two byte-granular stages (j = 16, 8) are one byte
// permute each with a per-lane selector, the three sub-byte stages one
// rotate (a funnel shift by a per-lane amount) and one masked merge each, so a
// stage is a shuffle plus one or two instructions.
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t transpose32(uint32_t x, int lane) {
    x = __byte_perm(x, __shfl_xor_sync(0xffffffffu, x, 16), (lane & 16) ? 0x3276u : 0x5410u);
    x = __byte_perm(x, __shfl_xor_sync(0xffffffffu, x, 8), (lane & 8) ? 0x3715u : 0x6240u);
#pragma unroll
    for (int j = 4; j > 0; j >>= 1) {
        const uint32_t m = j == 4 ? 0x0f0f0f0fu : j == 2 ? 0x33333333u : 0x55555555u;
        const bool hi = (lane & j) != 0;
        const uint32_t keep = hi ? ~m : m;                       // bits of x that stay
        const uint32_t y = __shfl_xor_sync(0xffffffffu, x, j);
        const uint32_t ys = __funnelshift_l(y, y, hi ? 32 - j : j);   // partner's bits moved into place
        x = (x & keep) | (ys & ~keep);
    }
    return x;
}

// x * 2^e, equal to ldexpf(x, e): a single multiplication by an exact power of
// two rounds once, as ldexpf does, whenever 2^e is a normal float
__device__ __forceinline__ float pow2f(int e) { return __int_as_float((e + 127) << 23); }
__device__ __forceinline__ bool pow2_normal(int e) { return e >= -126 && e <= 127; }
__device__ __forceinline__ float scale2(float v, int e, bool fast, float sc) { return fast ? v * sc : ldexpf(v, e); }

// (-2)^i as a float (exact)
__device__ __forceinline__ constexpr float nbw(int i) { return (i & 1) ? -(float)(1u << i) : (float)(1u << i); }


// asynchronous 4-byte global -> shared copies (cp.async), one group per call
__device__ __forceinline__ void cp_async4(uint32_t* dst, const uint32_t* src) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(d), "l"(src) : "memory");
}
// 16-byte copy, both addresses 16-byte aligned (L2 only)
__device__ __forceinline__ void cp_async16(uint32_t* dst, const uint32_t* src) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;\n" ::: "memory"); }

// The byte-granular second stage and the three sub-byte stages of a half
// transpose (below), on the 16 words the first stage selected.
__device__ __forceinline__ void transpose32_half_tail(uint32_t (&a)[16]) {
#pragma unroll
    for (int k = 0; k < 8; k++) {
        const uint32_t x = a[k], y = a[k + 8];
        a[k] = __byte_perm(x, y, 0x6240u);
        a[k + 8] = __byte_perm(x, y, 0x7351u);
    }
#pragma unroll
    for (int s = 0; s < 3; s++) {
        const int j = 4 >> s;
        const uint32_t m = s == 0 ? 0x0f0f0f0fu : s == 1 ? 0x33333333u : 0x55555555u;
#pragma unroll
        for (int i = 0; i < 8; i++) {
            const int k = (i / j) * 2 * j + (i % j);
            const uint32_t t = ((a[k] >> j) ^ a[k + j]) & m;
            a[k + j] ^= t;
            a[k] ^= t << j;
        }
    }
}

// Half of a 32 x 32 bit transpose: rows R[0..31] (R[r] bit e) -> the 16
// words out[v] (v = 16 * half + 0..15) whose bit r is R[r] bit v. The two
// byte-granular stages are byte permutes, the three sub-byte stages
// mask-and-shift swaps.
__device__ __forceinline__ void transpose32_half(const uint32_t (&R)[32], int half, uint32_t (&a)[16]) {
    const uint32_t sel16 = half ? 0x7632u : 0x5410u;
#pragma unroll
    for (int k = 0; k < 16; k++) a[k] = __byte_perm(R[k], R[k + 16], sel16);
    transpose32_half_tail(a);
}

constexpr int TB_LD = 36;   // block-major plane tile row: 32 planes + pad, 16-byte aligned rows

constexpr int NB_G = 8;              // blocks per warp iteration
constexpr int NB_CHUNK = 256;        // blocks per CTA chunk
constexpr int NB_TILE_LD = NB_CHUNK + 1;   // padded tile row: conflict-free column writes

// Encode chunk c (NB_CHUNK consecutive 32-value blocks) of a level: each warp
// transposes 32 blocks into the shared [plane][block] tile, then the CTA
// writes every plane's words of the chunk as one contiguous run
// (NegaBinaryBPEncoder.hpp:18-62). The error-table variant is in bitplane.cu.
// FULLB: B == 32, so every digit has a plane and no per-digit guard is needed
template <bool FULLB = false>
__device__ __forceinline__ void nb_encode32_chunk(const float* __restrict__ x, uint64_t n, uint64_t nblocks, int B,
                                                  int se, bool fast, float scale, uint32_t* __restrict__ out,
                                                  uint64_t stride, uint64_t c, uint32_t* tile) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int plane = B - 1 - lane;      // lane k owns bit k = plane B-1-k
    const uint64_t cb0 = c * NB_CHUNK;
    const uint64_t wb0 = cb0 + (uint64_t)warp * 32;
#pragma unroll 1
    for (int j0 = 0; j0 < 32; j0 += NB_G) {
        float v[NB_G];
#pragma unroll
        for (int g = 0; g < NB_G; g++) {
            const uint64_t i = (wb0 + j0 + g) * 32 + lane;
            v[g] = i < n ? __ldcs(x + i) : 0.f;
        }
#pragma unroll
        for (int g = 0; g < NB_G; g++) {
            // NegaBinaryBPEncoder.hpp:42; the scaling is chosen once per chunk
            // (an exact multiplication whenever 2^se is a normal float)
            const float sh = fast ? v[g] * scale : ldexpf(v[g], se);
            const uint32_t w = transpose32(nb_from_bin((int32_t)sh), lane);
            if (FULLB || lane < B) tile[plane * NB_TILE_LD + warp * 32 + j0 + g] = w;
        }
    }
    __syncthreads();
    const int nvalid = (int)((nblocks - cb0) < (uint64_t)NB_CHUNK ? (nblocks - cb0) : NB_CHUNK);
    for (int p = warp; p < B; p += 8) {
        uint32_t* dst = out + (uint64_t)p * stride + cb0;
        const uint32_t* row = tile + p * NB_TILE_LD;
        for (int j = lane; j < nvalid; j += 32) dst[j] = row[j];
    }
    __syncthreads();
}

// Decode chunk c of planes [s, s+num) (plane s+i at base + i * stride):
// coalesced tile load, one warp transpose per block, coalesced stores.
__device__ __forceinline__ void nb_decode32_chunk(const uint32_t* __restrict__ base, uint64_t stride, uint64_t n,
                                                  uint64_t nblocks, int num, int e, int exp, bool dfast, float dscale,
                                                  uint64_t c, uint32_t* tile, float* __restrict__ out) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const bool neg = num != 0 && (e & 1);                   // NegaBinaryBPEncoder.hpp:153, :177
    const uint64_t cb0 = c * NB_CHUNK;
    const int nvalid = (int)((nblocks - cb0) < (uint64_t)NB_CHUNK ? (nblocks - cb0) : NB_CHUNK);
    for (int p = warp; p < num; p += 8) {
        const uint32_t* src = base + (uint64_t)p * stride + cb0;
        uint32_t* row = tile + p * NB_TILE_LD;
        for (int j = lane; j < nvalid; j += 32) row[j] = __ldcs(src + j);
    }
    __syncthreads();
    for (int j = 0; j < 32; j++) {
        const int bl = warp * 32 + j;
        if (bl >= nvalid) break;
        const uint32_t w = lane < num ? tile[lane * NB_TILE_LD + bl] : 0u;
        const uint32_t col = transpose32(w, lane);      // bit i = digit of plane s+i
        const uint32_t a = num ? (__brev(col) >> (32 - num)) : 0u;
        const float val = num ? (dfast ? (float)nb_to_bin(a) * dscale : ldexpf((float)nb_to_bin(a), exp - e)) : 0.f;
        const uint64_t i = (cb0 + bl) * 32 + lane;
        if (i < n) out[i] = neg ? -val : val;
    }
    __syncthreads();
}

}  // namespace prodm
