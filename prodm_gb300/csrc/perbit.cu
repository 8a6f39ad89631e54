// Per-bit bitplane format on the device (sm_103a): PerBitBPEncoder
// (PerBitBPEncoder.hpp:7-146 encode, :290-383 progressive_decode).
//
// Reference stream format: one bit stream per plane, bits packed from the
// least significant end of 64-bit words. Element i writes, in plane p, bit
// (B-1-p) of its fixed-point magnitude and, right after its first 1 bit, its
// sign. Where a bit of plane p sits therefore depends on how many earlier
// elements had their first 1 bit in plane p: a stream can only be parsed with
// the planes before it.
//
// Device layout ("rows"): the level's elements in groups of 32; row p (p < B)
// holds one 32-bit word per group whose bit j is bit (B-1-p) of element
// 32g+j's magnitude; row B holds the sign words (bit j set: element negative
// and nonzero); row B+1 (parsed streams only) the elements that have no 1 bit
// in the planes parsed so far. Every row starts on a 16-byte boundary. In this
// layout decoding is a transpose per group and needs no parse; the reference
// stream sizes (ceil((n + first-ones in p) / 64) * 8 bytes) are computed at
// encode time, and pb_pack writes the reference streams on export.
#include "common.cuh"
#include "kernels.cuh"
#include "nbcodec.cuh"

namespace prodm {

namespace {

constexpr unsigned FULL = 0xffffffffu;
constexpr int PB_WARPS = 8;
constexpr int PB_GPW = 16;                        // groups per warp per chunk
constexpr int PB_CHUNK = PB_WARPS * PB_GPW;       // groups per CTA chunk
constexpr int PB_LD = PB_CHUNK + 1;               // padded tile row

template <class T>
__device__ __forceinline__ int pb_exp(const typename KeyOf<T>::type* maxkey, int exp_arg) {
    return maxkey ? frexp_exp(key_to_val(*maxkey, T())) : exp_arg;
}

// Fixed-point magnitude of one value, |trunc(ldexp(v, k))| with k = B - exp
// (PerBitBPEncoder.hpp:100-104). The scaling is exact (the result stays
// below 2^B), so the truncated magnitude is floor(|v| * 2^k): for doubles it
// is taken from the exponent and mantissa bits with integer operations
// (GB300's FP64 pipe is slow); for floats by one multiplication with an exact
// power of two where that is a normal float, else ldexpf.
__device__ __forceinline__ uint64_t pb_mag(double v, int k, bool, float) { return fixed_mag(v, k); }
__device__ __forceinline__ uint32_t pb_mag(float v, int k, bool fast, float sc) {
    return (uint32_t)fabsf(fast ? v * sc : ldexpf(v, k));
}
__device__ __forceinline__ bool pb_neg(double v) { return __double_as_longlong(v) < 0; }
__device__ __forceinline__ bool pb_neg(float v) { return v < 0.f; }

// ldexp((T)acc, s) (PerBitBPEncoder.hpp:343). For doubles with every result
// normal (fast: -1022 <= s <= 960), acc is rounded once to 53 bits (nearest,
// ties to even, as the conversion does) and the exponent field written
// directly; otherwise, and for floats, the conversion and an exact scaling.
__device__ __forceinline__ double pb_value(uint64_t acc, int s, bool fast, float) {
    return fast ? fixed_value(acc, s) : ldexp((double)acc, s);
}
__device__ __forceinline__ float pb_value(uint32_t acc, int s, bool fast, float sc) {
    return fast ? (float)acc * sc : ldexpf((float)acc, s);
}
__device__ __forceinline__ double pb_negate(double v) {
    return __longlong_as_double(__double_as_longlong(v) ^ (long long)0x8000000000000000ull);
}
__device__ __forceinline__ float pb_negate(float v) { return -v; }
__device__ __forceinline__ bool pb_value_fast(double*, int s) { return fixed_value_normal(s); }
__device__ __forceinline__ bool pb_value_fast(float*, int s) { return pow2_normal(s); }

__device__ __forceinline__ uint32_t valid_mask(int nvalid) { return nvalid >= 32 ? FULL : ((1u << nvalid) - 1u); }

// ---------------------------------------------------------------------------
// encode: values -> rows 0..B (magnitude planes + signs) and, per plane, the
// number of elements whose first 1 bit is in that plane
// ---------------------------------------------------------------------------
template <class T>
__global__ void __launch_bounds__(256) k_pb_encode(const T* __restrict__ x, uint64_t n,
                                                   const typename KeyOf<T>::type* __restrict__ maxkey, int exp_arg,
                                                   int B, uint32_t* __restrict__ rows, uint64_t stride,
                                                   uint32_t* __restrict__ counts) {
    using FP = typename Traits<T>::FP;
    extern __shared__ uint32_t tile[];   // (B + 1) rows x PB_LD
    __shared__ uint32_t cnt[64];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int exp = pb_exp<T>(maxkey, exp_arg);
    const int ks = B - exp;
    const bool fast = pow2_normal(ks);
    const float sc = fast ? pow2f(ks) : 1.f;
    const uint64_t ng = (n + 31) / 32;
    const uint64_t nch = (ng + PB_CHUNK - 1) / PB_CHUNK;
    for (int k = threadIdx.x; k < 64; k += blockDim.x) cnt[k] = 0;
    __syncthreads();
    for (uint64_t c = blockIdx.x; c < nch; c += gridDim.x) {
        const uint64_t g0 = c * PB_CHUNK;
#pragma unroll 2
        for (int j = 0; j < PB_GPW; j++) {
            const int gl = warp * PB_GPW + j;
            const uint64_t i = (g0 + gl) * 32 + lane;
            const T v = i < n ? __ldcs(x + i) : (T)0;
            const FP m = pb_mag(v, ks, fast, sc);
            const uint32_t sgn = __ballot_sync(FULL, pb_neg(v) && m != 0);
            // a value's first 1 bit is its most significant one: count the
            // group's values per msb (one shared atomic per distinct msb)
            const int msb = m ? (int)(8 * sizeof(FP)) - 1 - (sizeof(T) == 8 ? __clzll((long long)m) : __clz((int)m))
                              : -1;
            const unsigned same = __match_any_sync(FULL, msb);
            if (msb >= 0 && lane == __ffs(same) - 1) atomicAdd(&cnt[B - 1 - msb], (uint32_t)__popc(same));
            const uint32_t lo = transpose32((uint32_t)m, lane);          // lane k: bit k of the 32 magnitudes
            const uint32_t hi = sizeof(T) == 8 ? transpose32((uint32_t)((uint64_t)m >> 32), lane) : 0u;
            if (lane < B) tile[(B - 1 - lane) * PB_LD + gl] = lo;
            if (sizeof(T) == 8 && lane + 32 < B) tile[(B - 33 - lane) * PB_LD + gl] = hi;
            if (lane == 0) tile[B * PB_LD + gl] = sgn;
        }
        __syncthreads();
        const int nvalid = (int)((ng - g0) < (uint64_t)PB_CHUNK ? (ng - g0) : PB_CHUNK);
        for (int p = warp; p <= B; p += PB_WARPS) {
            uint32_t* dst = rows + (uint64_t)p * stride + g0;
            const uint32_t* src = tile + p * PB_LD;
            for (int j = lane; j < nvalid; j += 32) dst[j] = src[j];
        }
        __syncthreads();
    }
    __syncthreads();
    for (int p = threadIdx.x; p < B; p += blockDim.x)
        if (cnt[p]) atomicAdd(&counts[p], cnt[p]);
}

// reference stream sizes: BitEncoder words (n + first-one count bits) * 8
__global__ void k_pb_sizes(const uint32_t* __restrict__ counts, int B, uint64_t n, uint32_t* __restrict__ sizes) {
    const int p = threadIdx.x;
    if (p < B) sizes[p] = (uint32_t)((n + counts[p] + 63) / 64 * 8);
}

// ---------------------------------------------------------------------------
// decode planes [s, e): value = 2^(exp-e) * (magnitude bits of planes s..e-1),
// negative where the element's sign is known by plane e (progressive_decode
// :315-344: a sign is read with the first 1 bit) and its sign bit is set.
// `unseen` (row of elements without a 1 bit in planes < e) may be NULL when
// s == 0: then "known" is "nonzero". dnum (device plane count) overrides e.
// ---------------------------------------------------------------------------
// the groups of one staged chunk; FAST: every value is normal (no FP64 path
// in the loop)
template <class T, bool FAST>
__device__ __forceinline__ void pb_decode_groups(const uint32_t* tile, int num, int nvalid, uint64_t g0, uint64_t n,
                                                 int vs, float sc, bool with_unseen, T* __restrict__ out) {
    using FP = typename Traits<T>::FP;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll 2
    for (int j = 0; j < PB_GPW; j++) {
        const int gl = warp * PB_GPW + j;
        if (gl >= nvalid) break;
        const uint32_t wl = lane < num ? tile[(num - 1 - lane) * PB_LD + gl] : 0u;
        FP acc = transpose32(wl, lane);
        if (sizeof(T) == 8 && num > 32) {
            const uint32_t wh = lane + 32 < num ? tile[(num - 33 - lane) * PB_LD + gl] : 0u;
            acc |= (FP)((uint64_t)transpose32(wh, lane) << 32);
        }
        const uint32_t sg = tile[num * PB_LD + gl];
        const bool known = with_unseen ? !((tile[(num + 1) * PB_LD + gl] >> lane) & 1u) : acc != 0;
        const T v = pb_value(acc, vs, FAST, sc);
        const uint64_t i = (g0 + gl) * 32 + lane;
        if (i < n) out[i] = (known && ((sg >> lane) & 1u)) ? pb_negate(v) : v;
    }
}

template <class T>
__global__ void __launch_bounds__(256) k_pb_decode(const uint32_t* __restrict__ rows, uint64_t stride, uint64_t n,
                                                   const typename KeyOf<T>::type* __restrict__ maxkey, int exp_arg,
                                                   int s, int e, const uint8_t* __restrict__ dnum,
                                                   const uint32_t* __restrict__ srow,
                                                   const uint32_t* __restrict__ unseen, T* __restrict__ out) {
    extern __shared__ uint32_t tile[];   // num + 2 rows x PB_LD
    if (dnum) e = dnum[0];
    const int num = e - s;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int exp = pb_exp<T>(maxkey, exp_arg);
    const int vs = exp - e;
    const bool fast = pb_value_fast((T*)nullptr, vs);
    const float sc = (sizeof(T) == 4 && fast) ? pow2f(vs) : 1.f;
    const uint64_t ng = (n + 31) / 32;
    const uint64_t nch = (ng + PB_CHUNK - 1) / PB_CHUNK;
    const int extra = unseen ? 2 : 1;
    for (uint64_t c = blockIdx.x; c < nch; c += gridDim.x) {
        const uint64_t g0 = c * PB_CHUNK;
        const int nvalid = (int)((ng - g0) < (uint64_t)PB_CHUNK ? (ng - g0) : PB_CHUNK);
        for (int r = warp; r < num + extra; r += PB_WARPS) {
            const uint32_t* src = r < num ? rows + (uint64_t)(s + r) * stride + g0
                                          : (r == num ? srow + g0 : unseen + g0);
            uint32_t* dst = tile + r * PB_LD;
            for (int j = lane; j < nvalid; j += 32) dst[j] = __ldcs(src + j);
        }
        __syncthreads();
        if (fast) pb_decode_groups<T, true>(tile, num, nvalid, g0, n, vs, sc, unseen != nullptr, out);
        else pb_decode_groups<T, false>(tile, num, nvalid, g0, n, vs, sc, unseen != nullptr, out);
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// export: rows -> reference streams (BitEncoder layout), three passes
//   count: bits of every (plane, 256-group chunk)
//   scan:  chunk bit offsets within each plane
//   write: each group's segment of each plane (<= 64 bits) OR-ed into the
//          zeroed destination
// ---------------------------------------------------------------------------
constexpr int PK_T = 256;   // groups (threads) per chunk

__device__ __forceinline__ int pk_nvalid(uint64_t g, uint64_t ng, uint64_t n) {
    if (g >= ng) return 0;
    const uint64_t r = n - g * 32;
    return r < 32 ? (int)r : 32;
}

__global__ void __launch_bounds__(PK_T) k_pb_pack_count(const uint32_t* __restrict__ rows, uint64_t stride, uint64_t n,
                                                        int B, uint32_t* __restrict__ chunk_bits, uint64_t nch) {
    __shared__ uint32_t red[64];
    const int lane = threadIdx.x & 31;
    for (int k = threadIdx.x; k < 64; k += blockDim.x) red[k] = 0;
    __syncthreads();
    const uint64_t ng = (n + 31) / 32;
    const uint64_t g = (uint64_t)blockIdx.x * PK_T + threadIdx.x;
    const int nvalid = pk_nvalid(g, ng, n);
    const uint32_t vm = valid_mask(nvalid);
    uint32_t seen = 0;
    for (int p = 0; p < B; p++) {
        const uint32_t M = nvalid ? rows[(uint64_t)p * stride + g] & vm : 0u;
        const uint32_t F = M & ~seen;
        seen |= M;
        uint32_t bits = nvalid + __popc(F);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) bits += __shfl_xor_sync(FULL, bits, o);
        if (lane == 0 && bits) atomicAdd(&red[p], bits);
    }
    __syncthreads();
    for (int p = threadIdx.x; p < B; p += blockDim.x) chunk_bits[(uint64_t)p * nch + blockIdx.x] = red[p];
}

__global__ void k_pb_pack_scan(const uint32_t* __restrict__ chunk_bits, uint64_t nch, uint64_t* __restrict__ chunk_off) {
    const int lane = threadIdx.x;
    const uint64_t base = (uint64_t)blockIdx.x * nch;
    uint64_t run = 0;
    for (uint64_t c0 = 0; c0 < nch; c0 += 32) {
        const uint64_t c = c0 + lane;
        const uint64_t v = c < nch ? chunk_bits[base + c] : 0;
        uint64_t inc = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint64_t t = __shfl_up_sync(FULL, inc, o);
            if (lane >= o) inc += t;
        }
        if (c < nch) chunk_off[base + c] = run + inc - v;
        run += __shfl_sync(FULL, inc, 31);
    }
}

// segment of one group in one plane: magnitude bit of each element, with the
// sign bit inserted after each element whose first 1 bit is in the plane
__device__ __forceinline__ uint64_t pb_segment(uint32_t M, uint32_t F, uint32_t S) {
    uint64_t seg = M;
    uint32_t f = F;
    while (f) {   // highest first: the positions below stay in place
        const int j = 31 - __clz(f);
        f &= ~(1u << j);
        const uint64_t low = seg & ((2ull << j) - 1ull);
        const uint64_t high = seg >> (j + 1);
        seg = low | ((uint64_t)((S >> j) & 1u) << (j + 1)) | (high << (j + 2));
    }
    return seg;
}

__global__ void __launch_bounds__(PK_T) k_pb_pack_write(const uint32_t* __restrict__ rows, uint64_t stride, uint64_t n,
                                                        int B, const uint32_t* __restrict__ srow,
                                                        const uint64_t* __restrict__ chunk_off, uint64_t nch,
                                                        const uint32_t* __restrict__ sizes,
                                                        unsigned long long* __restrict__ dst) {
    __shared__ uint64_t base[64];
    __shared__ uint32_t wsum[PK_T / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (threadIdx.x == 0) {
        uint64_t a = 0;
        for (int p = 0; p < B; p++) { base[p] = a * 8; a += sizes[p]; }
    }
    __syncthreads();
    const uint64_t ng = (n + 31) / 32;
    const uint64_t g = (uint64_t)blockIdx.x * PK_T + threadIdx.x;
    const int nvalid = pk_nvalid(g, ng, n);
    const uint32_t vm = valid_mask(nvalid);
    const uint32_t S = nvalid ? srow[g] : 0u;
    uint32_t seen = 0;
    for (int p = 0; p < B; p++) {
        const uint32_t M = nvalid ? rows[(uint64_t)p * stride + g] & vm : 0u;
        const uint32_t F = M & ~seen;
        seen |= M;
        const uint32_t len = nvalid + __popc(F);
        uint32_t inc = len;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t t = __shfl_up_sync(FULL, inc, o);
            if (lane >= o) inc += t;
        }
        if (lane == 31) wsum[warp] = inc;
        __syncthreads();
        uint32_t woff = 0;
        for (int w = 0; w < warp; w++) woff += wsum[w];
        __syncthreads();
        if (len) {
            const uint64_t seg = pb_segment(M, F, S);
            const uint64_t off = base[p] + chunk_off[(uint64_t)p * nch + blockIdx.x] + woff + inc - len;
            const uint64_t w = off >> 6;
            const int sh = (int)(off & 63);
            atomicOr(dst + w, (unsigned long long)(seg << sh));
            if (sh && sh + (int)len > 64) atomicOr(dst + w + 1, (unsigned long long)(seg >> (64 - sh)));
        }
    }
}

// ---------------------------------------------------------------------------
// parse: reference streams of planes [a, a+np) -> rows a..a+np-1, with the
// unseen / sign rows carried from the planes before a and updated.
//
// One single-warp CTA per plane, all co-resident (cooperative launch). The
// chain over planes is a software pipeline over chunks of 32 groups: CTA k
// receives each chunk's unseen / sign masks from CTA k-1 through a ring in
// global memory (release / acquire flags) and hands them on after its plane.
// Within a chunk, only groups with unseen elements can hold sign bits: they
// are parsed in order, one step per sign bit (pz_group); the other groups
// hold exactly one bit per element, so once the sign bits before them are
// counted, every lane reads its group's word directly. Every wait is bounded: past the limit the CTA
// records PRODM_ETIMEOUT in *status and returns.
// ---------------------------------------------------------------------------
constexpr int PZ_R = 8;                      // ring depth (chunks)
constexpr long long kPzSpin = 1ll << 24;     // x >= 256 ns per wait

__device__ __forceinline__ int ld_acquire(const int* p) {
    int v;
    asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release(int* p, int v) {
    asm volatile("st.release.gpu.global.b32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// a plane's stream: the chunk's 64 64-bit words are staged in shared memory;
// the next chunk's are prefetched into registers n0 / n1 (lane i: words
// npb + i and npb + 32 + i)
struct PlaneReader {
    const uint64_t* w;
    uint64_t nw, pos, pb, npb;
    uint64_t n0, n1;
    __device__ __forceinline__ uint64_t load(uint64_t k) const { return k < nw ? __ldcs(w + k) : 0ull; }
};

__device__ __forceinline__ uint32_t bits_below(int k) { return k >= 32 ? FULL : ((1u << k) - 1u); }

// One group of one plane from the 64 stream bits W at its start. With d sign
// bits before them, the remaining elements' bits are the frame W >> d (bit i
// = element i); the next element to carry a sign is the lowest unseen one
// whose bit is set there, and its sign is bit i of the next frame W >> (d+1).
// One step per sign.
__device__ __forceinline__ void pz_group(uint64_t W, uint32_t U, int nv, uint32_t& M, uint32_t& SG, uint32_t& cnt) {
    const uint32_t lo32 = (uint32_t)W, hi32 = (uint32_t)(W >> 32);
    const uint32_t vm = bits_below(nv);
    uint32_t rest = U & vm, m = 0, sg = 0, below = 0, d = 0;
    uint32_t Wd = lo32;
    for (int it = 0; it < 33; it++) {
        const uint32_t T = rest & Wd;
        if (!T) break;
        const uint32_t bit = T & (0u - T);          // element i
        const uint32_t upto = (bit << 1) - 1u;      // elements 0..i
        m |= Wd & upto & ~below;
        below = upto;
        rest &= ~upto;
        d++;
        Wd = __funnelshift_rc(lo32, hi32, d);
        sg |= Wd & bit;
    }
    M = m | (Wd & vm & ~below);
    SG = sg;
    cnt = d;
}

// A group whose values are all unseen is a stream of the tokens "0" and
// "1 s": a 1 at a token start escapes the next bit. Runs of 1s start at token
// starts; inside a run the odd offsets are escaped, and the bit after a run
// of odd length is escaped too (the run-start parities split by adding the
// run starts: the carry clears a run and marks its end).
__device__ __forceinline__ uint64_t pz_escaped(uint64_t W) {
    constexpr uint64_t EVEN = 0x5555555555555555ull, ODD = 0xaaaaaaaaaaaaaaaaull;
    const uint64_t starts = W & ~(W << 1);
    const uint64_t es = W + (starts & EVEN), os = W + (starts & ODD);
    const uint64_t inside = ((W & ~es) & ODD) | ((W & ~os) & EVEN);
    const uint64_t after = ((es & ~W) & ODD) | ((os & ~W) & EVEN);
    return inside | after;
}
// position of zero number e (from 0) of E: binary search on popcounts
__device__ __forceinline__ int pz_select_zero(uint64_t E, int e) {
    const uint64_t Z = ~E;
    int pos = 0, rem = e;
#pragma unroll
    for (int step = 32; step > 0; step >>= 1) {
        const int c = __popcll((Z >> pos) & ((1ull << step) - 1ull));
        if (c <= rem) {
            rem -= c;
            pos += step;
        }
    }
    return pos;
}

// one chunk (32 groups, lane g = group g0 + g) of one plane; U / S: the
// lane's group's unseen and sign masks, updated; returns the group's word.
// ws: the chunk's stream as 128 32-bit words (word 2*pb + i at ws[i])
__device__ __forceinline__ uint32_t pz_chunk(PlaneReader& r, bool first, uint64_t g0, uint64_t ng, uint64_t n,
                                             uint32_t& U, uint32_t& S, int lane, uint32_t* ws, uint32_t* us,
                                             int* nvs) {
    // the chunk reads words [pos/64, pos/64 + 33); its successor starts 16..32
    // 64-bit words on (a full group takes 32..64 bits)
    const uint64_t wb = r.pos >> 6;
    __syncwarp();
    uint64_t a, b;
    if (first) {
        r.pb = wb;
        a = r.load(wb + lane);
        b = r.load(wb + 32 + lane);
    } else {
        r.pb = r.npb;
        a = r.n0;
        b = r.n1;
    }
    ws[2 * lane] = (uint32_t)a;
    ws[2 * lane + 1] = (uint32_t)(a >> 32);
    ws[64 + 2 * lane] = (uint32_t)b;
    ws[64 + 2 * lane + 1] = (uint32_t)(b >> 32);
    r.npb = wb + 16;
    r.n0 = r.load(r.npb + lane);
    r.n1 = r.load(r.npb + 32 + lane);
    const uint64_t g = g0 + lane;
    const int nv = pk_nvalid(g, ng, n);
    us[lane] = U;
    nvs[lane] = nv;
    __syncwarp();
    const uint32_t p0 = (uint32_t)(r.pos - 64 * r.pb);   // chunk start within the staged words (< 1088)
    uint32_t M = 0, extra = 0;
    // groups with unseen elements, in order (every lane computes the same):
    // the sign bits before group j are those of the earlier groups of this kind
    const uint32_t seq = __ballot_sync(FULL, nv > 0 && U != 0);
    uint32_t todo = seq, run = 0;
    while (todo) {
        const int j = __ffs(todo) - 1;
        todo &= todo - 1;
        const uint32_t Uj = us[j];
        const int nvj = nvs[j];
        const uint32_t at = p0 + 32u * j + run;
        const uint32_t k = at >> 5, sh = at & 31;
        const uint32_t x0 = ws[k], x1 = ws[k + 1], x2 = ws[k + 2];
        const uint64_t W = ((uint64_t)__funnelshift_r(x1, x2, sh) << 32) | __funnelshift_r(x0, x1, sh);
        uint32_t Mj, SG, cnt;
        if (Uj == bits_below(nvj)) {   // all unseen: bit-parallel, one value per lane
            const int q = pz_select_zero(pz_escaped(W), lane);
            const bool b = lane < nvj && ((W >> q) & 1ull);
            Mj = __ballot_sync(FULL, b);
            SG = __ballot_sync(FULL, b && ((W >> (q + 1)) & 1ull));
            cnt = __popc(Mj);
        } else {
            pz_group(W, Uj, nvj, Mj, SG, cnt);
        }
        const bool mine = lane == j;
        M = mine ? Mj : M;
        extra = mine ? cnt : extra;
        U = mine ? (Uj & ~Mj) : U;
        S = mine ? (S | SG) : S;
        run += cnt;
    }
    // groups without unseen elements: one bit per element at known offsets
    uint32_t inc = extra;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t t = __shfl_up_sync(FULL, inc, o);
        if (lane >= o) inc += t;
    }
    if (nv > 0 && !((seq >> lane) & 1u)) {
        const uint32_t at = p0 + 32u * lane + (inc - extra);
        M = __funnelshift_r(ws[at >> 5], ws[(at >> 5) + 1], at & 31) & valid_mask(nv);
    }
    uint32_t used = (uint32_t)nv;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) used += __shfl_xor_sync(FULL, used, o);
    r.pos += used + run;
    return M;
}

constexpr int PZ_SUB = 4;                    // 32-group sub-chunks per hand-off
constexpr int PZ_E = 64 * PZ_SUB;            // ring entry: unseen + sign words of 32 * PZ_SUB groups
// dynamic shared memory reserved (unused) so that no two planes' CTAs share an SM
constexpr int PZ_SPREAD_SMEM = 116 * 1024;

__global__ void __launch_bounds__(32) k_pb_parse(const uint64_t* const* __restrict__ planes,
                                                 const uint64_t* __restrict__ nwords, int a, int np, uint64_t n,
                                                 uint32_t* __restrict__ rows, uint64_t stride,
                                                 uint32_t* __restrict__ unseen, uint32_t* __restrict__ signs,
                                                 uint32_t* __restrict__ ring, int* __restrict__ flags,
                                                 int* __restrict__ status) {
    __shared__ uint32_t ws[130];
    __shared__ uint32_t us[32];
    __shared__ int nvs[32];
    const int k = blockIdx.x, lane = threadIdx.x;
    int* produced = flags;
    int* consumed = flags + np;
    const uint64_t ng = (n + 31) / 32, nch = (ng + 32 * PZ_SUB - 1) / (32 * PZ_SUB);
    PlaneReader r{planes[k], nwords[k], 0, 0, 0, 0, 0};
    uint32_t* row = rows + (uint64_t)(a + k) * stride;
    const bool last = k == np - 1;
    int seen_consumed = 0;   // the consumer's progress as last read
    for (uint64_t c = 0; c < nch; c++) {
        const int slot = (int)(c % PZ_R);
        uint32_t U[PZ_SUB], S[PZ_SUB];
        if (k == 0) {
#pragma unroll
            for (int t = 0; t < PZ_SUB; t++) {
                const uint64_t g = c * 32 * PZ_SUB + t * 32 + lane;
                U[t] = g < ng ? unseen[g] : 0u;
                S[t] = g < ng ? signs[g] : 0u;
            }
        } else {
            long long spins = 0;
            while (ld_acquire(produced + k - 1) <= (int)c) {
                if (++spins > kPzSpin) { if (lane == 0) atomicExch(status, PRODM_ETIMEOUT); return; }
                __nanosleep(128);
            }
            const uint32_t* src = ring + ((uint64_t)(k - 1) * PZ_R + slot) * PZ_E;
#pragma unroll
            for (int t = 0; t < PZ_SUB; t++) {
                U[t] = __ldcg(src + t * 64 + lane);
                S[t] = __ldcg(src + t * 64 + 32 + lane);
            }
            __syncwarp();
            if (lane == 0) st_release(consumed + k - 1, (int)c + 1);
        }
#pragma unroll
        for (int t = 0; t < PZ_SUB; t++) {
            const uint64_t g0 = c * 32 * PZ_SUB + t * 32;
            if (g0 >= ng) break;
            const uint32_t M = pz_chunk(r, c == 0 && t == 0, g0, ng, n, U[t], S[t], lane, ws, us, nvs);
            if (g0 + lane < ng) row[g0 + lane] = M;
        }
        if (last) {
#pragma unroll
            for (int t = 0; t < PZ_SUB; t++) {
                const uint64_t g = c * 32 * PZ_SUB + t * 32 + lane;
                if (g < ng) { unseen[g] = U[t]; signs[g] = S[t]; }
            }
        } else {
            if ((int)c - seen_consumed >= PZ_R) {
                long long spins = 0;
                while ((int)c - (seen_consumed = ld_acquire(consumed + k)) >= PZ_R) {
                    if (++spins > kPzSpin) { if (lane == 0) atomicExch(status, PRODM_ETIMEOUT); return; }
                    __nanosleep(128);
                }
            }
            uint32_t* dst = ring + ((uint64_t)k * PZ_R + slot) * PZ_E;
#pragma unroll
            for (int t = 0; t < PZ_SUB; t++) {
                __stcg(dst + t * 64 + lane, U[t]);
                __stcg(dst + t * 64 + 32 + lane, S[t]);
            }
            __syncwarp();
            if (lane == 0) {
                __threadfence();
                st_release(produced + k, (int)c + 1);
            }
        }
    }
    // a well-formed stream ends in its last word
    if (lane == 0 && (r.pos + 63) / 64 != r.nw) atomicCAS(status, 0, PRODM_ECORRUPT);
}

// unseen row of a fresh level: every element present
__global__ void k_pb_init_unseen(uint32_t* __restrict__ unseen, uint32_t* __restrict__ signs, uint64_t n) {
    const uint64_t ng = (n + 31) / 32;
    for (uint64_t g = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; g < ng; g += (uint64_t)gridDim.x * blockDim.x) {
        unseen[g] = valid_mask(pk_nvalid(g, ng, n));
        signs[g] = 0;
    }
}

}  // namespace

uint64_t pb_groups(uint64_t n) { return (n + 31) / 32; }
uint64_t pb_row_words(uint64_t n) { return (pb_groups(n) + 3) / 4 * 4; }

template <class T>
int launch_pb_encode(const T* x, uint64_t n, const void* maxkey, int exp, int B, uint32_t* rows, uint64_t stride,
                     uint32_t* counts, uint32_t* sizes, cudaStream_t st) {
    if (B < 1 || B > (sizeof(T) == 8 ? 63 : 32)) return fail(PRODM_EINVAL, "perbit: num_bitplanes out of range");
    PRODM_CUDA(cudaMemsetAsync(counts, 0, B * sizeof(uint32_t), st));
    const uint64_t nch = (pb_groups(n) + PB_CHUNK - 1) / PB_CHUNK;
    const size_t smem = (size_t)(B + 1) * PB_LD * 4;
    const unsigned grid = persistent_grid_for((const void*)k_pb_encode<T>, 256, smem, nch, 1u << 20);
    k_pb_encode<T><<<grid, 256, smem, st>>>(x, n, (const typename KeyOf<T>::type*)maxkey, exp, B, rows, stride, counts);
    PRODM_CHECK_LAUNCH("k_pb_encode");
    k_pb_sizes<<<1, 64, 0, st>>>(counts, B, n, sizes);
    PRODM_CHECK_LAUNCH("k_pb_sizes");
    return PRODM_OK;
}

template <class T>
int launch_pb_decode(const uint32_t* rows, uint64_t stride, uint64_t n, const void* maxkey, int exp, int B, int s, int e,
                     const uint8_t* dnum, const uint32_t* srow, const uint32_t* unseen, T* out, cudaStream_t st) {
    const int maxnum = dnum ? B : e - s;
    const size_t smem = (size_t)(maxnum + 2) * PB_LD * 4;
    const uint64_t nch = (pb_groups(n) + PB_CHUNK - 1) / PB_CHUNK;
    const unsigned grid = persistent_grid_for((const void*)k_pb_decode<T>, 256, smem, nch, 1u << 20);
    k_pb_decode<T><<<grid, 256, smem, st>>>(rows, stride, n, (const typename KeyOf<T>::type*)maxkey, exp, s, e, dnum,
                                            srow, unseen, out);
    PRODM_CHECK_LAUNCH("k_pb_decode");
    return PRODM_OK;
}

size_t pb_pack_scratch_bytes(uint64_t n, int B) {
    const uint64_t nch = (pb_groups(n) + PK_T - 1) / PK_T;
    return ((size_t)B * nch * (4 + 8) + 511) / 256 * 256;   // a multiple of 256 bytes
}

int launch_pb_pack(const uint32_t* rows, uint64_t stride, uint64_t n, int B, const uint32_t* sizes, uint64_t total,
                   uint8_t* dst, void* scratch, cudaStream_t st) {
    if ((uintptr_t)dst % 8) return fail(PRODM_EINVAL, "perbit pack: destination must be 8-byte aligned");
    const uint64_t nch = (pb_groups(n) + PK_T - 1) / PK_T;
    uint64_t* chunk_off = (uint64_t*)scratch;
    uint32_t* chunk_bits = (uint32_t*)(chunk_off + (uint64_t)B * nch);
    PRODM_CUDA(cudaMemsetAsync(dst, 0, total, st));
    if (nch == 0) return PRODM_OK;
    k_pb_pack_count<<<(unsigned)nch, PK_T, 0, st>>>(rows, stride, n, B, chunk_bits, nch);
    PRODM_CHECK_LAUNCH("k_pb_pack_count");
    k_pb_pack_scan<<<B, 32, 0, st>>>(chunk_bits, nch, chunk_off);
    PRODM_CHECK_LAUNCH("k_pb_pack_scan");
    k_pb_pack_write<<<(unsigned)nch, PK_T, 0, st>>>(rows, stride, n, B, rows + (uint64_t)B * stride, chunk_off, nch,
                                                    sizes, (unsigned long long*)dst);
    PRODM_CHECK_LAUNCH("k_pb_pack_write");
    return PRODM_OK;
}

int launch_pb_init_unseen(uint32_t* unseen, uint32_t* signs, uint64_t n, cudaStream_t st) {
    k_pb_init_unseen<<<grid_for(pb_groups(n), 256), 256, 0, st>>>(unseen, signs, n);
    PRODM_CHECK_LAUNCH("k_pb_init_unseen");
    return PRODM_OK;
}

size_t pb_parse_scratch_bytes(int np) { return (size_t)np * PZ_R * PZ_E * 4 + (size_t)2 * np * 4 + 256; }

int launch_pb_parse(const uint64_t* const* planes, const uint64_t* nwords, int a, int np, uint64_t n, uint32_t* rows,
                    uint64_t stride, uint32_t* unseen, uint32_t* signs, void* scratch, int* status, cudaStream_t st) {
    if (np < 1 || np > 64) return fail(PRODM_EINVAL, "perbit parse: 1..64 planes per call");
    uint32_t* ring = (uint32_t*)scratch;
    int* flags = (int*)(ring + (size_t)np * PZ_R * PZ_E);
    PRODM_CUDA(cudaMemsetAsync(flags, 0, (size_t)2 * np * 4, st));
    static thread_local int attr_dev = -1;
    int dev = 0;
    PRODM_CUDA(cudaGetDevice(&dev));
    if (attr_dev != dev) {
        PRODM_CUDA(cudaFuncSetAttribute((const void*)k_pb_parse, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        PZ_SPREAD_SMEM));
        attr_dev = dev;
    }
    // the planes' CTAs wait on one another: launched cooperatively, so that
    // all of them are resident together
    void* args[] = {(void*)&planes, (void*)&nwords, &a, &np, &n, &rows, &stride, &unseen, &signs, &ring, &flags,
                    &status};
    PRODM_CUDA(cudaLaunchCooperativeKernel((const void*)k_pb_parse, dim3(np), dim3(32), args, PZ_SPREAD_SMEM, st));
    PRODM_CHECK_LAUNCH("k_pb_parse");
    return PRODM_OK;
}

template int launch_pb_encode<float>(const float*, uint64_t, const void*, int, int, uint32_t*, uint64_t, uint32_t*,
                                     uint32_t*, cudaStream_t);
template int launch_pb_encode<double>(const double*, uint64_t, const void*, int, int, uint32_t*, uint64_t, uint32_t*,
                                      uint32_t*, cudaStream_t);
template int launch_pb_decode<float>(const uint32_t*, uint64_t, uint64_t, const void*, int, int, int, int,
                                     const uint8_t*, const uint32_t*, const uint32_t*, float*, cudaStream_t);
template int launch_pb_decode<double>(const uint32_t*, uint64_t, uint64_t, const void*, int, int, int, int,
                                      const uint8_t*, const uint32_t*, const uint32_t*, double*, cudaStream_t);

}  // namespace prodm
