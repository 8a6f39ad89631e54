// Layout conversion between the aligned device stream layout and the
// reference level-file bytes, plus small reductions (sm_103a).
//
// Reference level file (FileWriter.hpp:16-31 with NullLevelCompressor): the
// streams of planes 0..B-1 concatenated; for the grouped encoder stream 0 is
// [u32 nblocks][u8 rb x nblocks][words] (GroupedBPEncoder.hpp:370-377), so
// every later word may sit at any byte offset.
#include "common.cuh"
#include "kernels.cuh"

namespace prodm {

namespace {

template <class W>
__device__ __forceinline__ void store_bytes(uint8_t* dst, W w) {
    if (((uintptr_t)dst & (sizeof(W) - 1)) == 0) {
        *(W*)dst = w;
    } else {
#pragma unroll
        for (int i = 0; i < (int)sizeof(W); i++) dst[i] = (uint8_t)(w >> (8 * i));
    }
}
template <class W>
__device__ __forceinline__ W load_bytes(const uint8_t* src) {
    if (((uintptr_t)src & (sizeof(W) - 1)) == 0) return *(const W*)src;
    W w = 0;
#pragma unroll
    for (int i = 0; i < (int)sizeof(W); i++) w |= (W)src[i] << (8 * i);
    return w;
}

// one CTA row of threads per plane (blockIdx.y = plane)
template <class W>
__global__ void k_gr_pack(const W* const* __restrict__ planes, const uint32_t* __restrict__ sizes, int B,
                          uint64_t nblocks, const uint8_t* __restrict__ rbs, uint8_t* __restrict__ dst) {
    const int p = blockIdx.y;
    uint64_t off = 0;
    for (int q = 0; q < p; q++) off += sizes[q];
    uint64_t bytes = sizes[p];
    const uint64_t t0 = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x, ts = (uint64_t)gridDim.x * blockDim.x;
    if (p == 0) {
        uint64_t hdr = 4 + nblocks;
        for (uint64_t i = t0; i < hdr; i += ts) {
            uint8_t v;
            if (i < 4) v = (uint8_t)((uint32_t)nblocks >> (8 * i));
            else v = rbs[i - 4];
            dst[i] = v;
        }
        off += hdr;
        bytes -= hdr;
    }
    const uint64_t nw = bytes / sizeof(W);
    const W* src = planes[p];
    for (uint64_t w = t0; w < nw; w += ts) store_bytes<W>(dst + off + w * sizeof(W), src[w]);
}

template <class W>
__global__ void k_unpack_planes(const uint8_t* __restrict__ src, const uint64_t* __restrict__ src_off,
                                const uint64_t* __restrict__ nwords, W* const* __restrict__ dst) {
    const int p = blockIdx.y;
    const uint64_t nw = nwords[p];
    const uint8_t* s = src + src_off[p];
    W* d = dst[p];
    for (uint64_t w = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; w < nw; w += (uint64_t)gridDim.x * blockDim.x)
        d[w] = load_bytes<W>(s + w * sizeof(W));
}

template <class T>
__global__ void k_maxabs(const T* __restrict__ x, uint64_t n, typename KeyOf<T>::type* key) {
    using K = typename KeyOf<T>::type;
    K m = 0;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        K k = abs_key(x[i]);
        m = k > m ? k : m;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        K w = __shfl_xor_sync(0xffffffffu, m, o);
        m = w > m ? w : m;
    }
    if ((threadIdx.x & 31) == 0 && m) atomicMax(key, m);
}

// level error bound = max (x4 for negabinary, ComposedRefactor.hpp:111-112)
template <class T>
__global__ void k_bounds(const typename KeyOf<T>::type* __restrict__ keys, int nl, int negabinary, T* __restrict__ bounds) {
    int l = blockIdx.x * blockDim.x + threadIdx.x;
    if (l < nl) {
        T m = key_to_val(keys[l], T());
        bounds[l] = negabinary ? m * (T)4 : m;
    }
}

__global__ void k_fill_u32(uint32_t* dst, uint64_t n, uint32_t v) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        dst[i] = v;
}

}  // namespace

int launch_gr_pack(const void* const* planes, const uint32_t* sizes, int B, uint64_t nblocks, const uint8_t* rbs,
                   int word_bytes, uint8_t* dst, cudaStream_t st) {
    dim3 grid(device_sms(), B);
    if (word_bytes == 4) k_gr_pack<uint32_t><<<grid, 256, 0, st>>>((const uint32_t* const*)planes, sizes, B, nblocks, rbs, dst);
    else k_gr_pack<uint64_t><<<grid, 256, 0, st>>>((const uint64_t* const*)planes, sizes, B, nblocks, rbs, dst);
    PRODM_CHECK_LAUNCH("k_gr_pack");
    return PRODM_OK;
}

int launch_unpack_planes(const uint8_t* src, const uint64_t* src_off, const uint64_t* nwords, int nplanes,
                         int word_bytes, void* const* dst, uint64_t max_words, cudaStream_t st) {
    if (nplanes <= 0) return PRODM_OK;
    dim3 grid(grid_for(max_words, 256, 4), nplanes);
    if (word_bytes == 4) k_unpack_planes<uint32_t><<<grid, 256, 0, st>>>(src, src_off, nwords, (uint32_t* const*)dst);
    else k_unpack_planes<uint64_t><<<grid, 256, 0, st>>>(src, src_off, nwords, (uint64_t* const*)dst);
    PRODM_CHECK_LAUNCH("k_unpack_planes");
    return PRODM_OK;
}

template <class T>
int launch_maxabs(const T* x, uint64_t n, void* maxkey, cudaStream_t st) {
    k_maxabs<T><<<grid_for(n, 256, 8), 256, 0, st>>>(x, n, (typename KeyOf<T>::type*)maxkey);
    PRODM_CHECK_LAUNCH("k_maxabs");
    return PRODM_OK;
}

template <class T>
int launch_bounds_from_keys(const void* keys, int nl, int negabinary, T* bounds, cudaStream_t st) {
    k_bounds<T><<<1, 32, 0, st>>>((const typename KeyOf<T>::type*)keys, nl, negabinary, bounds);
    PRODM_CHECK_LAUNCH("k_bounds");
    return PRODM_OK;
}

int launch_fill_u32(uint32_t* dst, uint64_t n, uint32_t v, cudaStream_t st) {
    k_fill_u32<<<grid_for(n, 256, 4), 256, 0, st>>>(dst, n, v);
    PRODM_CHECK_LAUNCH("k_fill_u32");
    return PRODM_OK;
}

template int launch_maxabs<float>(const float*, uint64_t, void*, cudaStream_t);
template int launch_maxabs<double>(const double*, uint64_t, void*, cudaStream_t);
template int launch_bounds_from_keys<float>(const void*, int, int, float*, cudaStream_t);
template int launch_bounds_from_keys<double>(const void*, int, int, double*, cudaStream_t);

}  // namespace prodm
