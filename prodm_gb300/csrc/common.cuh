// Shared device/host helpers for the GB300 MDR kernels.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include <cstddef>
#include <string>

#include "../../include/prodm_gb300.h"

namespace prodm {

// ---------------------------------------------------------------------------
// error reporting (thread-local last error string for prodm_last_error_string)
// ---------------------------------------------------------------------------
void set_error(const std::string& msg);
int fail(int status, const std::string& msg);
int cuda_status(cudaError_t e, const char* where);

#define PRODM_CUDA(call)                                              \
    do {                                                              \
        cudaError_t _e = (call);                                      \
        if (_e != cudaSuccess) return ::prodm::cuda_status(_e, #call); \
    } while (0)
void count_launch();
#define PRODM_CHECK_LAUNCH(name)                                          \
    do {                                                                  \
        ::prodm::count_launch();                                          \
        cudaError_t _e = cudaGetLastError();                              \
        if (_e != cudaSuccess) return ::prodm::cuda_status(_e, name);     \
    } while (0)

// GB300's SM count (2 dies x 76): the fallback when the device cannot be
// queried and the basis of fixed buffer sizes (kPartialSlots); grids are
// sized from the current device's own count (device_sms)
constexpr int kSMs = 152;
int device_sms();   // multiprocessors of the current device (cached per device)

// ---------------------------------------------------------------------------
// Programmatic dependent launch along a chain of dependent kernels (one
// retrieval: interpreter -> multi-level decode -> level recompositions ->
// fused finest level). A kernel launched with launch_chain may start while
// its predecessor in the stream is still running; it calls pdl_wait() before
// touching anything the predecessor writes or reads, and pdl_release() only
// after that wait, so a kernel that starts early knows every kernel two or
// more launches back has completed. Both are no-ops for a normal launch.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_release() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }
bool pdl_enabled();   // false when the environment sets PRODM_NO_PDL=1

template <typename... KArgs, typename... Args>
cudaError_t launch_chain(bool pdl, void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t st,
                         Args... args) {
    if (!pdl || !pdl_enabled()) {
        kernel<<<grid, block, smem, st>>>(args...);
        return cudaGetLastError();
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kernel, static_cast<KArgs>(args)...);
}

// CTAs of `kernel` (threads, dynamic smem) resident on the whole current
// device at once: the grid of a persistent grid-stride kernel, so that no CTA
// waits for a second wave (cached per device, kernel and launch shape)
unsigned resident_ctas(const void* kernel, int threads, size_t smem);
inline unsigned persistent_grid_for(const void* kernel, int threads, size_t smem, uint64_t need, uint64_t max_grid) {
    uint64_t g = resident_ctas(kernel, threads, smem);
    if (g > need) g = need;
    if (g > max_grid) g = max_grid;
    return (unsigned)(g ? g : 1);
}

inline unsigned grid_for(size_t work, int threads, int per_sm = 8) {
    size_t g = (work + threads - 1) / threads;
    size_t cap = (size_t)device_sms() * per_sm;
    if (g > cap) g = cap;
    if (g == 0) g = 1;
    return (unsigned)g;
}

// ---------------------------------------------------------------------------
// Level geometry (3-D with leading unit dims for 1-D and 2-D fields).
// Every dim shrinks n -> (n >> 1) + 1 per level (RefactorUtils.hpp:21-34).
// ---------------------------------------------------------------------------
struct Box {
    uint32_t n[3];
    __host__ __device__ uint64_t size() const { return (uint64_t)n[0] * n[1] * n[2]; }
};

__host__ __device__ inline uint32_t coarse_len(uint32_t n) { return (n >> 1) + 1; }

// coarse nodes: even indices below n-1, plus n-1 itself
__host__ __device__ inline bool is_coarse(uint32_t x, uint32_t n) { return x == n - 1 || (x & 1u) == 0; }
__host__ __device__ inline uint32_t reord(uint32_t x, uint32_t n, uint32_t nc) {
    return is_coarse(x, n) ? (x == n - 1 ? nc - 1 : x >> 1) : nc + (x >> 1);
}
__host__ __device__ inline uint32_t fine_of_coarse(uint32_t m, uint32_t n, uint32_t nc) {
    return m == nc - 1 ? n - 1 : 2 * m;
}

// Position of reordered coordinate r in the interleaved order of the level
// box(F) \ box(C) (row-major walk that skips the coarse box,
// DirectInterleaver.hpp:23-31).
__host__ __device__ inline uint64_t level_rank(uint32_t r0, uint32_t r1, uint32_t r2, const Box& F, const Box& C) {
    uint64_t lin = ((uint64_t)r0 * F.n[1] + r1) * F.n[2] + r2;
    uint64_t pre = (uint64_t)min(r0, C.n[0]) * C.n[1] * C.n[2];
    if (r0 < C.n[0]) {
        pre += (uint64_t)min(r1, C.n[1]) * C.n[2];
        if (r1 < C.n[1]) pre += min(r2, C.n[2]);
    }
    return lin - pre;
}

struct LevelGeom {
    int ndims;
    int L;
    uint32_t dims[3];                  // as given (ndims entries)
    Box box[17];                       // padded 3-D box of each level (0..L)
    uint64_t elems[17];                // coefficients per level
    uint64_t offset[17];               // offset of each level in a packed coefficient array
    uint64_t total;
};
int make_geom(int ndims, const uint32_t* dims, int L, LevelGeom& g);
int max_level(int ndims, const uint32_t* dims);

// ---------------------------------------------------------------------------
// numeric helpers (exact operations only)
// ---------------------------------------------------------------------------
template <class T> struct Traits;
template <> struct Traits<float> {
    using S = uint32_t;    // stream word
    using FP = uint32_t;   // unsigned fixed point
    using FPS = int32_t;   // signed fixed point (negabinary source)
    using Bits = uint32_t;
    static constexpr int kBlock = 32;
    static constexpr int kPrec = 23;
};
template <> struct Traits<double> {
    using S = uint64_t;
    using FP = uint64_t;
    using FPS = int64_t;
    using Bits = uint64_t;
    static constexpr int kBlock = 64;
    static constexpr int kPrec = 52;
};

__device__ __forceinline__ uint32_t nb_from_bin(int32_t x) { return ((uint32_t)x + 0xaaaaaaaau) ^ 0xaaaaaaaau; }
__device__ __forceinline__ uint64_t nb_from_bin(int64_t x) {
    return ((uint64_t)x + 0xaaaaaaaaaaaaaaaaull) ^ 0xaaaaaaaaaaaaaaaaull;
}
__device__ __forceinline__ int32_t nb_to_bin(uint32_t x) { return (int32_t)((x ^ 0xaaaaaaaau) - 0xaaaaaaaau); }
__device__ __forceinline__ int64_t nb_to_bin(uint64_t x) {
    return (int64_t)((x ^ 0xaaaaaaaaaaaaaaaaull) - 0xaaaaaaaaaaaaaaaaull);
}

__device__ __forceinline__ int frexp_exp(float v) { int e; frexpf(v, &e); return e; }
__device__ __forceinline__ int frexp_exp(double v) { int e; frexp(v, &e); return e; }
__device__ __forceinline__ float ldexp_t(float v, int e) { return ldexpf(v, e); }
__device__ __forceinline__ double ldexp_t(double v, int e) { return ldexp(v, e); }

// floor(|v| * 2^k) of a double whose scaled magnitude stays below 2^63 (the
// encoders' |trunc(ldexp(v, k))|), from its exponent and mantissa bits with
// integer operations: GB300's FP64 pipe takes about two lane operations per
// SM cycle, too slow for a conversion per value
__device__ __forceinline__ uint64_t fixed_mag(double v, int k) {
    const uint64_t bits = (uint64_t)__double_as_longlong(v);
    const int ev = (int)((bits >> 52) & 0x7ff);
    uint64_t m = bits & 0xfffffffffffffull;
    int e = -1074;
    if (ev) {
        m |= 1ull << 52;
        e = ev - 1075;
    }
    const int sh = e + k;   // |v| * 2^k = m * 2^sh
    if (sh >= 0) return m << sh;
    return sh <= -64 ? 0ull : m >> (-sh);
}
// v < 0 for a double that is not NaN, without an FP64 comparison
__device__ __forceinline__ bool below_zero(double v) {
    const uint64_t bits = (uint64_t)__double_as_longlong(v);
    return (bits >> 63) && (bits << 1) != 0;
}
// ldexp((double)acc, s) for results that are normal (-1022 <= s <= 960): acc
// rounded once to 53 bits (nearest, ties to even, as the conversion does) and
// the exponent field written directly
__device__ __forceinline__ double fixed_value(uint64_t acc, int s) {
    if (acc == 0) return 0.0;
    const int msb = 63 - __clzll((long long)acc);
    int e2 = msb;
    uint64_t mant;
    if (msb <= 52) {
        mant = acc << (52 - msb);
    } else {
        const int sh = msb - 52;
        mant = acc >> sh;
        const uint64_t rem = acc & ((1ull << sh) - 1), half = 1ull << (sh - 1);
        if (rem > half || (rem == half && (mant & 1))) {
            mant++;
            if (mant >> 53) {
                mant >>= 1;
                e2++;
            }
        }
    }
    return __longlong_as_double((long long)(((uint64_t)(e2 + s + 1023) << 52) | (mant & 0xfffffffffffffull)));
}
__device__ __forceinline__ bool fixed_value_normal(int s) { return s >= -1022 && s <= 960; }

// uncontracted arithmetic (no FMA fusion), so that results match a host
// evaluation of the same expression tree operation by operation
__device__ __forceinline__ float add_rn(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double add_rn(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ float sub_rn(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ double sub_rn(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ float mul_rn(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }

// ---------------------------------------------------------------------------
// Column-pair form of the multilinear interpolation used by the row kernels.
// For a fine row (x0, x1) with odd-dim mask m01 over dims 0/1, the corner rows
// are: m01 = 0 -> 1 row; 1 -> (lo, hi) along dim 0; 2 -> (lo, hi) along dim 1;
// 3 -> (lo,lo), (lo,hi), (hi,lo), (hi,hi). q holds the corner values at one
// coarse column, qn those at the next coarse column. The even node of the
// column interpolates as tree(q); the odd node between the two columns as
// tree(avg(q, qn)): exactly the operation order of interp() (dim 0 outermost,
// dim 2 innermost), without lane divergence.
// ---------------------------------------------------------------------------
template <class T>
__device__ __forceinline__ T avg_rn(T a, T b) { return mul_rn((T)0.5, add_rn(a, b)); }
// x * 0.5 for doubles with integer operations (GB300's FP64 pipe is slow, its
// integer pipes idle in these kernels): while the result is normal the
// halving is exact and only the exponent field drops by one; zeros and
// subnormal results take the significand halved with ties to even (what the
// multiplication rounds to), Inf and NaN stay as they are
static __device__ __noinline__ double half_rare(double x) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    if (((b >> 52) & 0x7ffu) == 0x7ffu) return x;
    const unsigned long long sig = b & 0x1fffffffffffffull;   // hidden bit included when the field is 1
    const unsigned long long q = sig >> 1;
    return __longlong_as_double((long long)((b & 0x8000000000000000ull) | (q + (sig & q & 1ull))));
}
__device__ __forceinline__ double half_rn(double x) {
    const int hi = __double2hiint(x);
    const unsigned f = ((unsigned)hi >> 20) & 0x7ffu;
    if (f - 2u < 0x7fdu) return __hiloint2double(hi - 0x100000, __double2loint(x));
    return half_rare(x);
}
__device__ __forceinline__ double avg_rn(double a, double b) { return half_rn(__dadd_rn(a, b)); }
template <class T>
__device__ __forceinline__ T corner_tree(int m01, const T* q) {
    if (m01 == 0) return q[0];
    if (m01 != 3) return avg_rn(q[0], q[1]);
    return avg_rn(avg_rn(q[0], q[1]), avg_rn(q[2], q[3]));
}
template <class T>
__device__ __forceinline__ T corner_tree_mid(int m01, const T* q, const T* qn) {
    if (m01 == 0) return avg_rn(q[0], qn[0]);
    if (m01 != 3) return avg_rn(avg_rn(q[0], qn[0]), avg_rn(q[1], qn[1]));
    return avg_rn(avg_rn(avg_rn(q[0], qn[0]), avg_rn(q[1], qn[1])), avg_rn(avg_rn(q[2], qn[2]), avg_rn(q[3], qn[3])));
}
__host__ __device__ inline int corner_count(int m01) { return m01 == 0 ? 1 : (m01 == 3 ? 4 : 2); }

// 32 x 32 bit transpose held in one thread's registers: on exit a[k] bit e =
// bit k of the entry a[e] (five butterfly stages of 16 pair swaps)
__device__ __forceinline__ void transpose32_regs(uint32_t (&a)[32]) {
#pragma unroll
    for (int s = 0; s < 5; s++) {
        const int j = 16 >> s;
        const uint32_t m = s == 0 ? 0x0000ffffu : s == 1 ? 0x00ff00ffu : s == 2 ? 0x0f0f0f0fu : s == 3 ? 0x33333333u
                                                                                                     : 0x55555555u;
#pragma unroll
        for (int i = 0; i < 16; i++) {
            const int k = (i / j) * 2 * j + (i % j);
            const uint32_t t = ((a[k] >> j) ^ a[k + j]) & m;
            a[k + j] ^= t;
            a[k] ^= t << j;
        }
    }
}

// last segment whose first global item is <= g (segments sorted by `begin`)
template <class Seg>
__device__ __forceinline__ int find_seg(const Seg* segs, int nseg, uint64_t g, uint64_t Seg::*begin) {
    int lo = 0, hi = nseg - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (segs[mid].*begin <= g) lo = mid; else hi = mid - 1;
    }
    return lo;
}

// |x| of a non-negative float/double as an order-preserving unsigned key
__device__ __forceinline__ uint32_t abs_key(float v) { return __float_as_uint(v) & 0x7fffffffu; }
__device__ __forceinline__ unsigned long long abs_key(double v) {
    return (unsigned long long)__double_as_longlong(v) & 0x7fffffffffffffffull;
}
__device__ __forceinline__ float key_to_val(uint32_t k, float) { return __uint_as_float(k); }
__device__ __forceinline__ double key_to_val(unsigned long long k, double) { return __longlong_as_double((long long)k); }
template <class T> struct KeyOf { using type = uint32_t; };
template <> struct KeyOf<double> { using type = unsigned long long; };

}  // namespace prodm
