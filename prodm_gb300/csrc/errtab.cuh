// Exact squared-error tables of the fp32 negabinary and grouped encoders
// (NegaBinaryBPEncoder.hpp:65-125 with collect_level_errors :231-239;
// GroupedBPEncoder.hpp:76-145 with collect_level_errors :324-335).
//
// The reference sums, in double and value by value, for every value x of a
// level (x = the value scaled by 2^(B - exp), a float):
//   entry B-k (k = 1..B-1) : (r_k + m)^2, r_k = integer value of the k low
//                            digits, m = x - trunc(x) (the fraction);
//   entry 0                : fl(x * x)  (a float product);
//   entry B                : fl(m * m) (negabinary) or m * m (grouped).
// Here every table is an exact integer computation, independent of the order
// in which values are visited, followed by one conversion to double:
//
// * With t = trunc(x) + 0xAAAAAAAA (negabinary; so t = nb ^ 0xAAAAAAAA) or
//   t = trunc(|x|) (grouped, A = 0), r_k = (t mod 2^k) - A_k with
//   A_k = A mod 2^k, so  sum r_k^2 = sum u_k^2 - 2 A_k sum u_k + n A_k^2
//   (u_k = t mod 2^k). sum u_k is sum_{b<k} 2^b * (count of bit b of t), the
//   popcounts of the transposed plane words. sum u_k^2 splits t into bytes
//   t_0..t_3: for k = 8J + s, u_k = u_{8J} + 2^{8J} h (h = t_J mod 2^s) and
//   u_k^2 = u_{8J}^2 + 2^{8J+1} sum_{j<J} 2^{8j} t_j h + 2^{16J} h^2, so the
//   byte products sum t_j h and sum h^2 are all that is accumulated: four
//   values at a time with __dp4a into 76 exact 32-bit lane sums.
// * |x| >= 2^23: x is an integer, m = 0, and fl(x^2) is an integer multiple of
//   2^23 below 2^65 (accumulated exactly as fl(x^2) / 2^23).
// * 1 <= |x| < 2^23: m = M * 2^-23 with an integer M, and
//   (r_k + m)^2 = r_k^2 + 2^-22 r_k M + 2^-46 M^2: the cross sums
//   sum u_k M = sum_{b<k} 2^b sum_{bit b of t} M and sum M^2 are exact
//   integers; so are the float-rounded squares the reference adds for
//   entries 0 and B: fl(x^2) * 2^23 (below 2^69) and fl(m^2) * 2^46 (below
//   2^46). |x| < 1: r_k = 0, m = x, x^2 is exact in double and fl(x^2) is
//   summed in double. These values (about 5 % of a 32-plane level) are
//   queued per warp and handled 32 at a time: one lane per value for their
//   own terms, then one lane per bit b of t for the masked sums.
// * The only doubles (the |x| < 1 terms, rare) are summed per lane and
//   reduced in a fixed order, so every table is bitwise reproducible.
#pragma once
#include "common.cuh"

namespace prodm {
namespace errtab {

// per-CTA record (u64 words), one per (CTA, level); 128-bit sums as lo, hi
constexpr int SQ = 0;       // 31: sum h_{J,s}^2, slot k-1 for k = 8J + s
constexpr int CR = 31;      // 45: sum t_j h_{J,s} (j < J), slot cr_slot(j, J, s)
constexpr int PC = 76;      // 32: count of bit b of t over the CTA's values
constexpr int S6A = 108;    // u128: sum fl(x^2) / 2^23 over |x| >= 2^23
constexpr int X = 110;      // 31 x i128: Y_b = sum of M over 1 <= |x| < 2^23 with bit b of t, slot X + 2b
constexpr int S4 = 172;     // u128: sum M^2
constexpr int SM = 174;     // i128: sum M
constexpr int S5 = 176;     // double: sum x^2 over |x| < 1
constexpr int STINY = 177;  // double: sum fl(x^2) over |x| < 1 (= sum fl(m^2) there)
constexpr int S6B = 178;    // u128: sum fl(x^2) * 2^23 over 1 <= |x| < 2^23
constexpr int S7B = 180;    // u128: sum fl(m^2) * 2^46 over 1 <= |x| < 2^23 (negabinary entry B)
constexpr int WORDS = 182;
constexpr int kSlotsPad = 200;   // WORDS + 2 x 8 warps of flush scratch, padded

// how the final reduction sums slot i: 0 = u64, 1 = low word of a 128-bit
// sum (its high word follows), 2 = high word, 3 = double
__host__ __device__ constexpr int slot_kind(int i) {
    return (i >= S6A && i < S5) || (i >= S6B && i < WORDS) ? (((i - (i >= S6B ? S6B : S6A)) & 1) ? 2 : 1)
           : (i == S5 || i == STINY) ? 3 : 0;
}

__host__ __device__ constexpr int cr_slot(int j, int J, int s) {
    return J == 1 ? (s - 1) : J == 2 ? 8 + 8 * j + (s - 1) : 24 + 7 * j + (s - 1);
}

constexpr int kRing = 256;   // per-warp queue of values with |x| < 2^23

// per-warp shared state of the queue side (one lane's sums per slot)
struct WarpQ {
    float ring[kRing];
    uint2 batch[32];          // (t, M) of the batch being processed
    unsigned long long s4[32];
    long long sm[32];
    unsigned long long xlo[32];
    long long xhi[32];
    unsigned long long s6lo[32], s6hi[32], s7[32];
    double s5[32], stiny[32];
};

// per-lane register sums
struct Lane {
    uint32_t sq[31];
    uint32_t cr[45];
    uint32_t pc;              // popcount of this lane's plane words (bit = lane)
    unsigned long long s6a;   // sum fl(x^2) / 2^23 over |x| >= 2^23

    __device__ __forceinline__ void zero() {
#pragma unroll
        for (int i = 0; i < 31; i++) sq[i] = 0;
#pragma unroll
        for (int i = 0; i < 45; i++) cr[i] = 0;
        pc = 0;
        s6a = 0;
    }

    // four values' t (any order: the sums are symmetric in the values)
    __device__ __forceinline__ void add4(uint32_t t0, uint32_t t1, uint32_t t2, uint32_t t3) {
        const uint32_t x01 = __byte_perm(t0, t1, 0x5140u), y01 = __byte_perm(t0, t1, 0x7362u);
        const uint32_t x23 = __byte_perm(t2, t3, 0x5140u), y23 = __byte_perm(t2, t3, 0x7362u);
        uint32_t P[4];
        P[0] = __byte_perm(x01, x23, 0x5410u);   // byte 0 of the four values
        P[1] = __byte_perm(x01, x23, 0x7632u);   // byte 1
        P[2] = __byte_perm(y01, y23, 0x5410u);   // byte 2
        P[3] = __byte_perm(y01, y23, 0x7632u);   // byte 3
#pragma unroll
        for (int J = 0; J < 4; J++) {
#pragma unroll
            for (int s = 1; s <= 8; s++) {
                const int k = 8 * J + s;
                if (k <= 31) {
                    const uint32_t H = s == 8 ? P[J] : (P[J] & (0x01010101u * ((1u << s) - 1u)));
                    sq[k - 1] = __dp4a(H, H, sq[k - 1]);
#pragma unroll
                    for (int j = 0; j < J; j++) cr[cr_slot(j, J, s)] = __dp4a(P[j], H, cr[cr_slot(j, J, s)]);
                }
            }
        }
    }

    // fl(x^2) / 2^23 when big (|x| >= 2^23: x^2 >= 2^46 rounds to a multiple
    // of 2^23, at most 2^64, so the scaled product is an integer below 2^42:
    // its significand shifted by the exponent - 46); no branch
    __device__ __forceinline__ void add_big_square(float x, bool big) {
        const uint32_t b = __float_as_uint(__fmul_rn(x, x));
        const uint32_t mant = (b & 0x7fffffu) | 0x800000u;
        const uint32_t sh = ((b >> 23) - 173u) & 31u;   // biased exponent - 127 - 46, in [0, 18] when big
        const unsigned long long v = (unsigned long long)mant << sh;
        s6a += big ? v : 0ull;
    }
};

__device__ __forceinline__ void add128(unsigned long long& lo, long long& hi, long long v) {
    const unsigned long long o = lo;
    lo += (unsigned long long)v;
    hi += (v < 0 ? -1ll : 0ll) + (lo < o ? 1ll : 0ll);
}

__device__ __forceinline__ void zero_q(WarpQ& q, int lane) {
    q.s4[lane] = 0;
    q.sm[lane] = 0;
    q.xlo[lane] = 0;
    q.xhi[lane] = 0;
    q.s6lo[lane] = 0;
    q.s6hi[lane] = 0;
    q.s7[lane] = 0;
    q.s5[lane] = 0;
    q.stiny[lane] = 0;
}

// fl(x^2) * 2^23 for 1 <= |x| < 2^23 as (lo, hi): the float square is in
// [1, 2^46), its significand shifted left by its exponent (0..45)
__device__ __forceinline__ void square_2p23(float x, unsigned long long& lo, unsigned long long& hi) {
    const uint32_t b = __float_as_uint(__fmul_rn(x, x));
    const unsigned long long mant = (b & 0x7fffffu) | 0x800000u;
    const int sh = (int)(b >> 23) - 127;
    lo = mant << sh;
    hi = sh ? mant >> (64 - sh) : 0ull;
}

// fl(m^2) * 2^46 for a fraction m = M * 2^-23, |M| < 2^23: zero, or a float
// in [2^-46, 1) whose value times 2^46 is an integer (the significand
// shifted by its exponent - 104, in -23..22; a right shift drops zeros only)
__device__ __forceinline__ unsigned long long frac_square_2p46(float m) {
    const uint32_t b = __float_as_uint(__fmul_rn(m, m));
    const unsigned long long mant = (b & 0x7fffffu) | 0x800000u;
    const int sh = (int)(b >> 23) - 104;
    return b == 0 ? 0ull : (sh >= 0 ? mant << sh : mant >> -sh);
}

// Process cnt (<= 32) queued values starting at ring slot head. NB: values are
// the signed scaled values; grouped: their magnitudes. Lane e takes value e's
// own terms; then lane b adds the M of the batch's values whose t has bit b
// set (Y_b; the cross sums are sum_k u_k M = sum_{b<k} 2^b Y_b). Entries past
// cnt are (0, 0) and add nothing.
template <bool NB>
__device__ __forceinline__ void run_batch(WarpQ& q, uint32_t head, int cnt, int lane) {
    int32_t M = 0;
    uint32_t t = 0;
    if (lane < cnt) {
        const float x = q.ring[(head + lane) & (kRing - 1)];
        const int32_t iq = (int32_t)x;                       // |x| < 2^23
        const float m = __fsub_rn(x, (float)iq);             // exact fraction
        t = NB ? (uint32_t)iq + 0xaaaaaaaau : (uint32_t)iq;
        if (fabsf(x) >= 1.f) {
            M = (int32_t)(m * 8388608.f);                     // exact: m is a multiple of 2^-23
            q.s4[lane] += (unsigned long long)((long long)M * M);
            q.sm[lane] += M;
            unsigned long long lo, hi;
            square_2p23(x, lo, hi);
            const unsigned long long o = q.s6lo[lane];
            q.s6lo[lane] = o + lo;
            q.s6hi[lane] += hi + (o + lo < o ? 1ull : 0ull);
            if (NB) q.s7[lane] += frac_square_2p46(m);
        } else {                                              // m = x
            q.s5[lane] += (double)x * (double)x;              // exact in double
            q.stiny[lane] += (double)__fmul_rn(x, x);
        }
    }
    q.batch[lane] = make_uint2(t, (uint32_t)M);
    __syncwarp();
    int32_t y = 0;                                            // |y| < 32 * 2^23
#pragma unroll
    for (int e2 = 0; e2 < 32; e2++) {
        const uint2 b = q.batch[e2];
        if ((b.x >> lane) & 1u) y += (int32_t)b.y;
    }
    add128(q.xlo[lane], q.xhi[lane], y);
    __syncwarp();
}

// Queue the values of one four-value step whose flag is set (|x| < 2^23) in
// one pass: the four ballots give each value its ring slot, the stores are
// predicated, and no branch depends on the data. qn is warp-uniform.
__device__ __forceinline__ void enqueue4(WarpQ& q, uint32_t head, int& qn, const bool (&small)[4],
                                         const float (&v)[4], int lane) {
    const uint32_t lt = (1u << lane) - 1u;
    uint32_t pos = head + (uint32_t)qn;
#pragma unroll
    for (int g = 0; g < 4; g++) {
        const uint32_t bal = __ballot_sync(0xffffffffu, small[g]);
        if (small[g]) q.ring[(pos + __popc(bal & lt)) & (kRing - 1)] = v[g];
        pos += __popc(bal);
    }
    qn = (int)(pos - head);
}

template <bool NB>
__device__ __forceinline__ void drain_full(WarpQ& q, uint32_t& head, int& qn, int lane) {
    if (qn >= 32) {
        __syncwarp();
        do {
            run_batch<NB>(q, head, 32, lane);
            head += 32;
            qn -= 32;
        } while (qn >= 32);
    }
}

// Add this CTA's sums (lanes' registers and every warp's queue sums; the queue
// must be empty) into its record; every thread of the CTA calls it. Integer
// parts are exact whatever the order; doubles are summed in a fixed order.
// red: kSlotsPad u64 of shared memory.
__device__ __forceinline__ void flush(Lane& a, WarpQ* wq, unsigned long long* red, unsigned long long* rec) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int i = threadIdx.x; i < kSlotsPad; i += blockDim.x) red[i] = 0;
    __syncthreads();
    // register sums: warp totals (u64), then shared atomics (integers: any order)
#pragma unroll
    for (int i = 0; i < 76; i++) {
        unsigned long long v = i < 31 ? a.sq[i] : a.cr[i - 31];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == 0) atomicAdd(&red[i], v);
    }
    atomicAdd(&red[PC + lane], (unsigned long long)a.pc);
    {
        // lane sums of fl(x^2) / 2^23 (< 2^42 each) as 128-bit warp totals in
        // the free slots after WORDS (two per warp)
        unsigned long long lo = a.s6a, hi = 0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const unsigned long long l2 = __shfl_xor_sync(0xffffffffu, lo, o), h2 = __shfl_xor_sync(0xffffffffu, hi, o);
            const unsigned long long ol = lo;
            lo += l2;
            hi += h2 + (lo < ol ? 1 : 0);
        }
        if (lane == 0) { red[WORDS + 2 * warp] = lo; red[WORDS + 2 * warp + 1] = hi; }
    }
    __syncthreads();
    if (threadIdx.x < 31) {            // Y_b, b = threadIdx.x: 128-bit over warps
        unsigned long long lo = 0;
        long long hi = 0;
        for (int w = 0; w < nw; w++) {
            const unsigned long long o = lo;
            lo += wq[w].xlo[threadIdx.x];
            hi += wq[w].xhi[threadIdx.x] + (lo < o ? 1 : 0);
        }
        unsigned long long* r = rec + X + 2 * threadIdx.x;
        const unsigned long long o = r[0];
        r[0] = o + lo;
        r[1] = (unsigned long long)((long long)r[1] + hi + ((o + lo) < o ? 1 : 0));
    } else if (threadIdx.x == 32) {    // fixed-order double sums, 128-bit integer sums
        double s5 = 0, st = 0;
        unsigned long long s4lo = 0, s4hi = 0, smlo = 0, s6lo = 0, s6hi = 0, s7lo = 0, s7hi = 0;
        long long smhi = 0;
        for (int w = 0; w < nw; w++)
            for (int l = 0; l < 32; l++) {
                s5 += wq[w].s5[l];
                st += wq[w].stiny[l];
                unsigned long long o = s4lo;
                s4lo += wq[w].s4[l];
                s4hi += s4lo < o ? 1 : 0;
                add128(smlo, smhi, wq[w].sm[l]);
                o = s6lo;
                s6lo += wq[w].s6lo[l];
                s6hi += wq[w].s6hi[l] + (s6lo < o ? 1 : 0);
                o = s7lo;
                s7lo += wq[w].s7[l];
                s7hi += s7lo < o ? 1 : 0;
            }
        rec[S5] = __double_as_longlong(__longlong_as_double(rec[S5]) + s5);
        rec[STINY] = __double_as_longlong(__longlong_as_double(rec[STINY]) + st);
        auto add_u128 = [&](int slot, unsigned long long lo, unsigned long long hi) {
            const unsigned long long o = rec[slot];
            rec[slot] = o + lo;
            rec[slot + 1] += hi + (rec[slot] < o ? 1 : 0);
        };
        add_u128(S4, s4lo, s4hi);
        add_u128(S6B, s6lo, s6hi);
        add_u128(S7B, s7lo, s7hi);
        const unsigned long long o = rec[SM];
        rec[SM] = o + smlo;
        rec[SM + 1] = (unsigned long long)((long long)rec[SM + 1] + smhi + (rec[SM] < o ? 1 : 0));
    }
    // u64 register sums and the S6A total (its high word stays for carries)
    for (int i = threadIdx.x; i < PC + 32; i += blockDim.x) rec[i] += red[i];
    if (threadIdx.x == 64) {
        unsigned long long lo = rec[S6A], hi = rec[S6A + 1];
        for (int w = 0; w < nw; w++) {
            const unsigned long long o = lo;
            lo += red[WORDS + 2 * w];
            hi += red[WORDS + 2 * w + 1] + (lo < o ? 1 : 0);
        }
        rec[S6A] = lo;
        rec[S6A + 1] = hi;
    }
    __syncthreads();
    zero_q(wq[warp], lane);
    a.zero();
    __syncthreads();
}

// ---------------------------------------------------------------------------
// final tables: sum the CTA records of a level and convert
// ---------------------------------------------------------------------------
__device__ __forceinline__ double u128_to_double(unsigned __int128 v) {
    return (double)(unsigned long long)(v >> 64) * 18446744073709551616.0 + (double)(unsigned long long)v;
}
__device__ __forceinline__ double i128_to_double(__int128 v) {
    return v < 0 ? -u128_to_double((unsigned __int128)(-v)) : u128_to_double((unsigned __int128)v);
}
__device__ __forceinline__ unsigned __int128 rd_u128(const unsigned long long* p) {
    return ((unsigned __int128)p[1] << 64) | p[0];
}

// Table of one level from the summed record R (u64 words), n values, B
// planes, exponent e (negabinary: the level exponent + 2); entry i of out.
template <bool NB>
__device__ double table_entry(const unsigned long long* R, uint64_t n, int B, int e, int i) {
    const uint32_t A = NB ? 0xaaaaaaaau : 0u;
    double v;
    if (i == 0) {   // (S6A * 2^46 + S6B) * 2^-23: one exact 128-bit sum
        v = u128_to_double((rd_u128(R + S6A) << 46) + rd_u128(R + S6B)) * 0x1p-23 + __longlong_as_double(R[STINY]);
    } else if (i == B) {
        v = NB ? u128_to_double(rd_u128(R + S7B)) * 0x1p-46 + __longlong_as_double(R[STINY])
               : u128_to_double(rd_u128(R + S4)) * 0x1p-46 + __longlong_as_double(R[S5]);
    } else {
        const int k = B - i;
        // sum u_k^2 from the byte products
        unsigned __int128 su2 = 0;
        for (int J = 0; 8 * J < k; J++) {
            const int s = k - 8 * J < 8 ? k - 8 * J : 8;
            if (8 * J + s < k) {   // a whole byte below k: u_{8(J+1)}^2 builds on it
                unsigned __int128 t = (unsigned __int128)R[SQ + 8 * J + 8 - 1] << (16 * J);
                for (int j = 0; j < J; j++) t += (unsigned __int128)R[CR + cr_slot(j, J, 8)] << (8 * (j + J) + 1);
                su2 += t;
            } else {
                unsigned __int128 t = (unsigned __int128)R[SQ + k - 1] << (16 * J);
                for (int j = 0; j < J; j++) t += (unsigned __int128)R[CR + cr_slot(j, J, s)] << (8 * (j + J) + 1);
                su2 += t;
            }
        }
        unsigned __int128 su = 0;
        for (int b = 0; b < k; b++) {
            const unsigned long long cb = ((A >> b) & 1u) ? n - R[PC + b] : R[PC + b];
            su += (unsigned __int128)cb << b;
        }
        const unsigned __int128 ak = (unsigned __int128)(k == 32 ? A : (A & ((1u << k) - 1u)));
        const __int128 sr2 = (__int128)su2 - (__int128)(2 * ak * su) + (__int128)(ak * ak * n);
        __int128 xk = -(__int128)ak * (__int128)rd_u128(R + SM);       // sum r_k M = sum u_k M - A_k sum M
        for (int b = 0; b < k; b++) xk += (__int128)rd_u128(R + X + 2 * b) << b;
        v = i128_to_double(sr2) + i128_to_double(xk) * 0x1p-22 + u128_to_double(rd_u128(R + S4)) * 0x1p-46 +
            __longlong_as_double(R[S5]);
    }
    return ldexp(v, 2 * (e - B));
}

}  // namespace errtab
}  // namespace prodm
