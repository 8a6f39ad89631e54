// Greedy size interpreters and error estimators on the device (sm_103a).
//
// Restates GreedyBasedSizeInterpreter.hpp:28-64 (greedy), :78-140
// (sign-exclude) and :166-248 (negabinary look-ahead) together with the
// estimators of MaxErrorEstimator.hpp:13-68 and SquaredErrorEstimator.hpp:
// 12-68. The estimators compute in the data type T exactly as the reference
// templates do, and the max-heap follows the sift order of the C++ standard
// library's priority_queue, so ties resolve identically. One thread runs one
// interpretation (one field); the kernel takes all inputs from device memory
// so a whole retrieval can run without a host round trip.
#include <climits>

#include "common.cuh"
#include "kernels.cuh"

namespace prodm {

namespace {

constexpr int kMaxLevels = 17;

// level factor of the L2 / S-norm estimators (SquaredErrorEstimator.hpp:12-68):
// 2^(ndims (L - i)), or 2^(2 s i + ndims (L - i)); the integer power is exact
template <class T>
__device__ T est_level_factor(int k, int ndims, int L, double s, int i) {
    if (k == 2) return (T)ldexp(1.0, ndims * (L - i));
    const T sT = (T)s;
    return (T)exp2((double)(2 * sT * i + ndims * (L - i)));
}

template <class T>
struct DevEstimator {
    int kind;
    T c;
    const T* table;    // per-level factors (shared memory), kinds 2 and 3
    __device__ void init(int k, int ndims, const T* tab) {
        kind = k;
        c = 0;
        table = tab;
        if (k == 1) {
            double cc = ndims == 1 ? 1.0 + sqrt(3.0) / 2 : ndims == 2 ? 1.0 + 9.0 / 4 : 1.0 + 21.0 * sqrt(3.0) / 8;
            c = (T)cc;
            c *= 4;
        }
    }
    __device__ T est(T e, int l) const {
        switch (kind) {
            case 0: return e;
            case 1: return c * e;
            case 2: return table[l] * e * (T)2;
            default: return table[l] * e;
        }
    }
    __device__ T gain(T cur, T next, int l) const {
        switch (kind) {
            case 0: return cur - next;
            case 1: return c * (cur - next);
            default: return table[l] * (cur - next);
        }
    }
};

// A heap entry carries its efficiency as an order-preserving integer key
// (equal doubles -> equal keys, +0 and -0 included) and a NaN flag, so the
// heap's `a.u < b.u` is evaluated with integer compares: every comparison
// with a NaN is false, as for the doubles.
struct Item { long long key; int nan; int level; int num; };

__device__ __forceinline__ void eff_key(double u, long long& key, int& nan) {
    const long long bits = __double_as_longlong(u);
    const long long mag = bits & 0x7fffffffffffffffll;
    nan = mag > 0x7ff0000000000000ll;
    key = mag == 0 ? 0 : (bits >= 0 ? bits : (bits ^ 0x7fffffffffffffffll));
}

struct DevHeap {
    Item h[kMaxLevels + 1];
    int len;
    __device__ static bool less(const Item& a, const Item& b) { return !(a.nan | b.nan) && a.key < b.key; }
    __device__ void sift_up(int hole, int top, Item v) {
        int parent = (hole - 1) / 2;
        while (hole > top && less(h[parent], v)) { h[hole] = h[parent]; hole = parent; parent = (hole - 1) / 2; }
        h[hole] = v;
    }
    __device__ void push(Item v) { h[len] = v; len++; sift_up(len - 1, 0, v); }
    __device__ void pop() {
        if (len > 1) {
            Item v = h[len - 1];
            h[len - 1] = h[0];
            int n = len - 1, hole = 0, child = 0;
            while (child < (n - 1) / 2) {
                child = 2 * (child + 1);
                if (less(h[child], h[child - 1])) child--;
                h[hole] = h[child];
                hole = child;
            }
            if ((n & 1) == 0 && child == (n - 2) / 2) {
                child = 2 * (child + 1);
                h[hole] = h[child - 1];
                hole = child - 1;
            }
            sift_up(hole, 0, v);
        }
        len--;
    }
};

// Efficiency of taking planes starting at index idx of level l. Every
// estimator ignores its base argument, so this depends on (l, idx) only and is
// tabulated once per call by the whole CTA.
//   kinds 0 / 1: gain(E[idx], E[idx+1]) / sizes[idx]
//   kind 2:      estimated_efficiency (GreedyBasedSizeInterpreter.hpp:228-248),
//                the look-ahead over consecutive planes with u32 size sums
template <class T>
__device__ void eff_entry(int kind, const DevEstimator<T>& est, int B, const uint32_t* sizes, const double* errs, int l,
                          int idx, double& u, int& num) {
    auto E = [&](int lv, int j) { return errs[(size_t)lv * (B + 1) + j]; };
    auto S = [&](int lv, int j) { return sizes[(size_t)lv * B + j]; };
    double cg = est.gain((T)E(l, idx), (T)E(l, idx + 1), l);
    uint32_t cs = S(l, idx);
    double ce = cg / cs;
    int cn = 1;
    if (kind == 2) {
        for (int i = 2; i < B - idx; i++) {
            double ng = est.gain((T)E(l, idx), (T)E(l, idx + i), l);
            uint32_t ns = cs + S(l, idx + i - 1);
            double ne = ng / ns;
            if ((ce > 0) && (ce > ne)) break;
            cg = ng;
            ce = ne;
            cs = ns;
            cn = i;
        }
    }
    u = ce;
    num = cn;
}

// ev[l * 65 + j] = (double) estimator(errors[l][j], l), tabulated by the CTA
// (the reference converts the estimator's T result to double on every use)
__device__ void interpret_core(int kind, int nl, int B, const uint32_t* __restrict__ sizes,
                               const double* __restrict__ ev, const long long* __restrict__ ekey,
                               const int8_t* __restrict__ enan, const int8_t* __restrict__ en, double tol,
                               uint8_t* index, uint32_t* rsz) {
    auto EST = [&](int l, int j) { return ev[l * 65 + j]; };
    auto S = [&](int l, int j) { return sizes[(size_t)l * B + j]; };
    auto item = [&](int l, int j) { return Item{ekey[l * 64 + j], (int)enan[l * 64 + j], l, (int)en[l * 64 + j]}; };
    for (int i = 0; i < nl; i++) rsz[i] = 0;
    double acc = 0;
    for (int i = 0; i < nl; i++) acc += EST(i, index[i]);
    DevHeap heap;
    heap.len = 0;
    if (kind == 0) {
        // a fully retrieved level has no next plane (the reference would read
        // past its error table here); it is not pushed
        for (int i = 0; i < nl; i++)
            if (index[i] != B) heap.push(item(i, index[i]));
        bool met = false;
        while (!met && heap.len > 0) {
            Item t = heap.h[0];
            heap.pop();
            int i = t.level, j = index[i];
            rsz[i] += S(i, j);
            acc -= EST(i, j);
            acc += EST(i, j + 1);
            if (acc < tol) met = true;
            index[i]++;
            if (index[i] != B) heap.push(item(i, index[i]));
        }
        return;
    }
    if (kind == 1) {
        if (acc < tol) return;
        double minerr = acc;
        for (int i = 0; i < nl; i++) {
            minerr -= EST(i, index[i]);
            minerr += EST(i, B);
            if (index[i] == 0) {
                rsz[i] += S(i, 0);
                acc -= EST(i, 0);
                acc += EST(i, 1);
                index[i]++;
            }
            if (index[i] != B) heap.push(item(i, index[i]));
            if (minerr < tol) break;
        }
        bool met = acc < tol;
        while (!met && heap.len > 0) {
            Item t = heap.h[0];
            heap.pop();
            int i = t.level, j = index[i];
            rsz[i] += S(i, j);
            acc -= EST(i, j);
            acc += EST(i, j + 1);
            if (acc < tol) met = true;
            index[i]++;
            if (index[i] != B) heap.push(item(i, index[i]));
        }
        return;
    }
    for (int i = 0; i < nl; i++)
        if (index[i] != B) heap.push(item(i, index[i]));
    bool met = acc < tol;
    if (met) return;
    while (!met && heap.len > 0) {
        Item t = heap.h[0];
        heap.pop();
        int i = t.level, j = index[i], num = t.num;
        for (int k = 0; k < num; k++) rsz[i] += S(i, j + k);
        acc -= EST(i, j);
        acc += EST(i, j + num);
        if (acc < tol) met = true;
        index[i] += num;
        if (index[i] != B) heap.push(item(i, index[i]));
    }
}

// The same walk with one lane per level. While every efficiency in the heap
// is a number and the largest one is unique, a max-heap pops exactly the
// largest entry, so the pop order is the arg-max order over the levels' next
// entries and the heap's layout does not matter. The warp tracks that
// condition at every pop; when it fails (a NaN efficiency -- zero-size
// planes -- or a tie for the maximum) it returns false and the caller runs
// the exact heap simulation from the original inputs. The estimate `acc` is
// updated in the same order by every lane.
__device__ bool interpret_warp(int kind, int nl, int B, const uint32_t* __restrict__ sizes,
                               const double* __restrict__ ev, const long long* __restrict__ ekey,
                               const int8_t* __restrict__ enan, const int8_t* __restrict__ en, double tol,
                               uint8_t* index, uint32_t* rsz, int lane) {
    const unsigned FULLM = 0xffffffffu;
    const bool has = lane < nl;
    int idx = has ? index[lane] : 0;
    uint32_t rs = 0;
    double acc = 0;
    for (int i = 0; i < nl; i++) acc += ev[i * 65 + index[i]];
    bool in_heap = has && idx != B;
    bool met = false;
    if (kind == 1) {
        if (acc < tol) {
            if (has) rsz[lane] = 0;
            return true;
        }
        double minerr = acc;
        in_heap = false;
        for (int i = 0; i < nl; i++) {
            const int ii = index[i];
            minerr -= ev[i * 65 + ii];
            minerr += ev[i * 65 + B];
            int ni = ii;
            if (ii == 0) {
                acc -= ev[i * 65 + 0];
                acc += ev[i * 65 + 1];
                ni = 1;
                if (lane == i) { rs += sizes[(size_t)i * B]; idx = 1; }
            }
            if (lane == i) in_heap = ni != B;
            if (minerr < tol) break;
        }
        met = acc < tol;
    } else if (kind == 2) {
        met = acc < tol;
    }
    while (!met) {
        long long k = LLONG_MIN;
        int nan = 0, num = 1;
        if (in_heap) {
            k = ekey[lane * 64 + idx];
            nan = enan[lane * 64 + idx];
            num = en[lane * 64 + idx];
        }
        if (!__any_sync(FULLM, in_heap)) break;
        if (__any_sync(FULLM, in_heap && nan)) return false;
        // arg-max of the 64-bit keys: unsigned order-preserving halves, two warp reductions
        const unsigned long long uk = (unsigned long long)k ^ 0x8000000000000000ull;
        const unsigned hi = (unsigned)(uk >> 32), lo = (unsigned)uk;
        const unsigned best_hi = __reduce_max_sync(FULLM, in_heap ? hi : 0u);
        const bool cand = in_heap && hi == best_hi;
        const unsigned best_lo = __reduce_max_sync(FULLM, cand ? lo : 0u);
        const unsigned at = __ballot_sync(FULLM, cand && lo == best_lo);
        if (__popc(at) != 1) return false;
        const int w = __ffs(at) - 1;
        const int j = __shfl_sync(FULLM, idx, w);
        const int take = __shfl_sync(FULLM, num, w);
        if (lane == w) {
            for (int t = 0; t < take; t++) rs += sizes[(size_t)lane * B + j + t];
            idx += take;
            in_heap = idx != B;
        }
        acc -= ev[w * 65 + j];
        acc += ev[w * 65 + j + take];
        if (acc < tol) met = true;
    }
    if (has) {
        index[lane] = (uint8_t)idx;
        rsz[lane] = rs;
    }
    return true;
}

// The same walk with the pop order computed in parallel. A level's entries
// (its chain: idx, idx + num, ..) fall into blocks: a block starts at an
// entry whose efficiency is below every earlier one of the level (the first
// entry starts one) and runs until the next such entry. When the largest
// head is unique at every pop, a popped block start is larger than every
// other head, and the rest of its block is at least as large, so a block
// leaves the heap in one run, and blocks leave in decreasing order of their
// start efficiency. So the pop order is the blocks sorted by start key, each
// in chain order; a pop meets a tie exactly when it starts a block whose key
// another level's block shares (tied blocks are ordered by level and flag
// their first entry). Thread 0 then runs the estimate `acc` along that order
// in the reference's arithmetic (two dependent double adds per pop, eight
// pops per round before their comparisons), stopping at the first estimate
// below the tolerance. Returns false -- nothing written -- when an
// efficiency is NaN or the walk reaches a tie before it stops; the caller
// then runs the walks above. All threads of the CTA call it.
// x (a finite double) as a signed integer count of 2^elsb, truncated toward
// zero (off by less than one unit); |x| < 2^(elsb + 114) keeps the shift
// below 61 bits and the result below 2^114
__device__ __forceinline__ __int128 fixed_units(double x, int elsb) {
    const uint64_t b = (uint64_t)__double_as_longlong(x);
    const int ev = (int)((b >> 52) & 0x7ff);
    uint64_t m = b & 0xfffffffffffffull;
    int e = -1074;   // |x| = m * 2^e
    if (ev) {
        m |= 1ull << 52;
        e = ev - 1075;
    }
    const int sh = e - elsb;
    const __int128 v = sh >= 0 ? (__int128)m << sh : (sh <= -64 ? (__int128)0 : (__int128)(m >> -sh));
    return (b >> 63) ? -v : v;
}
__device__ __forceinline__ int exp_field(double x) { return (int)(((uint64_t)__double_as_longlong(x) >> 52) & 0x7ff); }
// an upper bound of |v| / 2^80 (at least 1; below 2^46 for |v| < 2^125)
__device__ __forceinline__ uint64_t mag_units80(__int128 v) {
    const unsigned __int128 a = (unsigned __int128)(v < 0 ? -v : v);
    return (uint64_t)(a >> 80) + 1;
}

constexpr int kFixK = 5;   // positions per thread in the fixed-point pass (256 threads cover 17 x 64)

__device__ __forceinline__ __int128 shfl_up128(__int128 x, int o) {
    const unsigned long long lo = __shfl_up_sync(0xffffffffu, (unsigned long long)x, o);
    const unsigned long long hi = __shfl_up_sync(0xffffffffu, (unsigned long long)((unsigned __int128)x >> 64), o);
    return (__int128)(((unsigned __int128)hi << 64) | lo);
}
// exclusive prefix over the CTA's threads (in thread order) of one value per
// thread: warp scans by shuffles, then the warp totals; tot: one slot per warp
__device__ __int128 cta_exclusive_scan(__int128 v, __int128* tot) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    __int128 x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const __int128 y = shfl_up128(x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) tot[wid] = x;
    __syncthreads();
    if (wid == 0) {
        __int128 t = lane < nw ? tot[lane] : (__int128)0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const __int128 y = shfl_up128(t, o);
            if (lane >= o) t += y;
        }
        if (lane < nw) tot[lane] = t;
    }
    __syncthreads();
    const __int128 off = wid > 0 ? tot[wid - 1] : (__int128)0;
    __syncthreads();   // the slots may be reused right after
    return off + x - v;
}

struct BlockWalkSmem {
    uint8_t ch_j[kMaxLevels][64];      // chain entries of each level (plane index)
    uint16_t order[kMaxLevels * 64];   // pop order: level << 8 | plane index
    uint8_t tie[kMaxLevels * 64];      // 1: the pop at this position starts a tied block
    // every level's blocks in one list (levels in any order): level | entry
    // count << 16 | first entry << 24 (their keys in the caller's blk_key)
    uint32_t binfo[kMaxLevels * 64];
    int lat[kMaxLevels], lnb[kMaxLevels];   // each level's blocks: [lat, lat + lnb) of the list, keys falling
    uint32_t rs[kMaxLevels];
    int nidx[kMaxLevels];
    uint8_t start[kMaxLevels], n_ent[kMaxLevels], in_heap[kMaxLevels];
    int nblk, npos, fail, met0, stop;
    double acc0;
    // the fixed-point pass: largest exponent field, per-thread totals for the
    // scans, first positions (certainly met, undecided, tie)
    int maxev, first_met, first_amb, first_tie, fixed_ok;
    __int128 tot[32];   // one per warp (scans)
};

__device__ bool interpret_blocks(int kind, int nl, int B, const uint32_t* __restrict__ sizes,
                                 const double* __restrict__ ev, const long long* __restrict__ ekey,
                                 const int8_t* __restrict__ enan, const int8_t* __restrict__ en, double tol,
                                 uint8_t* index, uint32_t* rsz, long long* blk_key /* [kMaxLevels][64] */,
                                 BlockWalkSmem& w) {
    const int tid = threadIdx.x, nth = blockDim.x;
    // initial estimate, the sign-exclude first planes, heap membership
    if (tid == 0) {
        double acc = 0;
        for (int i = 0; i < nl; i++) acc += ev[i * 65 + index[i]];
        bool met = false;
        w.fail = 0;
        for (int i = 0; i < nl; i++) {
            w.start[i] = index[i];
            w.rs[i] = 0;
            w.in_heap[i] = kind != 1 && index[i] != B;
        }
        if (kind == 1) {
            if (acc < tol) {
                met = true;   // nothing retrieved, nothing pushed
            } else {
                double minerr = acc;
                for (int i = 0; i < nl; i++) {
                    const int ii = index[i];
                    minerr -= ev[i * 65 + ii];
                    minerr += ev[i * 65 + B];
                    int ni = ii;
                    if (ii == 0) {
                        acc -= ev[i * 65 + 0];
                        acc += ev[i * 65 + 1];
                        ni = 1;
                        w.rs[i] = sizes[(size_t)i * B];
                        w.start[i] = 1;
                    }
                    w.in_heap[i] = ni != B;
                    if (minerr < tol) break;
                }
                met = acc < tol;
            }
        } else if (kind == 2) {
            met = acc < tol;
        }
        w.met0 = met;
        w.acc0 = acc;
        w.nblk = 0;
        w.npos = 0;
    }
    __syncthreads();
    // each level's chain and blocks (one thread per level), the blocks into
    // one shared list
    uint8_t* lfirst = reinterpret_cast<uint8_t*>(w.order);   // [kMaxLevels][64]: first entry of each block
    if (tid < nl) {
        const int l = tid;
        int cnt = 0, nb = 0;
        if (w.in_heap[l]) {
            long long runmin = 0;
            for (int j = w.start[l]; j < B; j += en[l * 64 + j]) {
                const long long k = ekey[l * 64 + j];
                if (enan[l * 64 + j]) w.fail = 1;
                if (cnt == 0 || k < runmin) {
                    lfirst[l * 64 + nb++] = (uint8_t)cnt;
                    runmin = k;
                }
                w.ch_j[l][cnt++] = (uint8_t)j;
            }
        }
        w.n_ent[l] = (uint8_t)cnt;
        w.lnb[l] = nb;
        w.lat[l] = 0;
        if (nb) {   // the level's blocks into the shared list: key (its first entry's) and info
            atomicAdd(&w.npos, cnt);
            const int at = atomicAdd(&w.nblk, nb);
            w.lat[l] = at;
            for (int b = 0; b < nb; b++) {
                const int f0 = lfirst[l * 64 + b], f1 = b + 1 < nb ? lfirst[l * 64 + b + 1] : cnt;
                blk_key[at + b] = ekey[l * 64 + w.ch_j[l][f0]];
                w.binfo[at + b] = (uint32_t)l | (uint32_t)(f1 - f0) << 16 | (uint32_t)f0 << 24;
            }
        }
    }
    __syncthreads();
    if (w.fail) return false;
    // rank of each block: the entries of every block with a larger key, or an
    // equal key at a lower level (a tie, flagged). Its own level's earlier
    // blocks are the entries before it there; in every other level the
    // blocks' keys fall strictly, so a binary search finds the first block
    // whose key is not larger, and that block's first entry is the count.
    const int nblk = w.nblk;
    for (int t = tid; t < nblk; t += nth) {
        const uint32_t bi = w.binfo[t];
        const int l = bi & 255;
        const long long k = blk_key[t];
        int rank = (int)(bi >> 24);
        bool tie = false;
        for (int l2 = 0; l2 < nl; l2++) {
            const int nb2 = w.lnb[l2];
            if (l2 == l || nb2 == 0) continue;
            const int base = w.lat[l2];
            int lo = 0, hi = nb2;
            while (lo < hi) {
                const int mid = (lo + hi) >> 1;
                if (blk_key[base + mid] > k) lo = mid + 1;
                else hi = mid;
            }
            int first = lo;
            if (lo < nb2 && blk_key[base + lo] == k) {
                tie = true;
                if (l2 < l) first = lo + 1;   // the lower level's tied block goes first
            }
            rank += first < nb2 ? (int)(w.binfo[base + first] >> 24) : (int)w.n_ent[l2];
        }
        const int f0 = bi >> 24, n = (bi >> 16) & 255;
        for (int e = 0; e < n; e++) {
            w.order[rank + e] = (uint16_t)(l << 8 | w.ch_j[l][f0 + e]);
            w.tie[rank + e] = (uint8_t)(tie && e == 0);
        }
    }
    __syncthreads();
    // each pop's two estimate terms as indices into ev (the block list is
    // free again): ev[lo] leaves the estimate, ev[hi] enters it
    uint32_t* terms = w.binfo;
    for (int p = tid; p < w.npos; p += nth) {
        const int o = w.order[p], l = o >> 8, j = o & 255;
        terms[p] = (uint32_t)(l * 65 + j) | (uint32_t)(l * 65 + j + en[l * 64 + j]) << 16;
    }
    __syncthreads();
    // The stop from exact prefix sums (all threads). With R_p the exact sum
    // acc0 + sum_{i<=p} (add_i - sub_i) and R'_p = R_{p-1} - sub_p, the
    // reference's rounded estimate differs from R_p by at most
    // E_p = 2^-52 sum_{i<=p} (|R'_i| + |R_i|) (each double add rounds by at most
    // 2^-53 of its result; the factor 2 covers the compounding). The sums run
    // in 128-bit fixed point (unit 2^-113 of the largest value, truncations
    // counted in the bound); a position is certainly met when R_p + E_p is
    // below the tolerance, certainly not when R_p - E_p is above it. The stop
    // is the first certain one when nothing undecided comes before it; a tie
    // reached first bails out; an undecided position (the estimate within
    // rounding of the tolerance) leaves the decision to the sequential walk
    // below, as does a non-finite value or a tolerance that is not positive.
    const int np = w.npos;
    if (tid == 0) {
        w.maxev = max(exp_field(w.acc0), exp_field(tol));
        w.first_met = w.first_amb = w.first_tie = np;
        w.fixed_ok = !w.met0 && tol > 0.0 && np > 0;
    }
    __syncthreads();
    for (int p = tid; p < np; p += nth) {
        const uint32_t tq = terms[p];
        atomicMax(&w.maxev, max(exp_field(ev[tq & 0xffffu]), exp_field(ev[tq >> 16])));
    }
    __syncthreads();
    if (w.fixed_ok && w.maxev < 0x7ff) {
        const int elsb = (w.maxev - 1022 + 1) + 12 - 125;   // all |values| < 2^(maxev - 1022 + 1); 2^11 pops of headroom
        const int p0 = tid * kFixK;
        __int128 rr[kFixK], rp[kFixK];
        __int128 dsum = 0;
#pragma unroll
        for (int u = 0; u < kFixK; u++) {
            rr[u] = rp[u] = 0;
            if (p0 + u < np) {
                const uint32_t tq = terms[p0 + u];
                const __int128 a = fixed_units(ev[tq & 0xffffu], elsb), b = fixed_units(ev[tq >> 16], elsb);
                rp[u] = -a;   // R'_p - R_{p-1} for now
                rr[u] = b - a;
                dsum += b - a;
            }
        }
        __int128 run = fixed_units(w.acc0, elsb) + cta_exclusive_scan(dsum, w.tot);   // R_{p0 - 1}
        uint64_t usum = 0, uu[kFixK];
#pragma unroll
        for (int u = 0; u < kFixK; u++) {
            uu[u] = 0;
            if (p0 + u < np) {
                rp[u] += run;    // R'_p
                run += rr[u];    // R_p
                rr[u] = run;
                uu[u] = mag_units80(rp[u]) + mag_units80(rr[u]);
                usum += uu[u];
            }
        }
        uint64_t srun = (uint64_t)cta_exclusive_scan((__int128)usum, w.tot);
        const __int128 tfix = fixed_units(tol, elsb);
        int fm = np, fa = np, ft = np;
#pragma unroll
        for (int u = 0; u < kFixK; u++) {
            const int p = p0 + u;
            if (p >= np) break;
            srun += uu[u];
            const __int128 e = ((__int128)srun << 28) + 2 * p + 4;   // in units; 2^-52 * 2^80 = 2^28
            if (w.tie[p] && ft == np) ft = p;
            if (rr[u] + e < tfix) {
                if (fm == np) fm = p;
            } else if (!(rr[u] - e >= tfix + 1)) {
                if (fa == np) fa = p;
            }
        }
        if (fm < np) atomicMin(&w.first_met, fm);
        if (fa < np) atomicMin(&w.first_amb, fa);
        if (ft < np) atomicMin(&w.first_tie, ft);
    } else if (tid == 0) {
        w.fixed_ok = 0;
    }
    __syncthreads();
    // the sequential estimate (thread 0) where the fixed-point pass left the
    // decision open: each round loads eight pops' terms, runs the two
    // dependent double adds per pop, then compares the eight estimates with
    // the tolerance
    if (tid == 0) {
        int stop = np;   // pops [0, stop)
        bool bail = false;
        const int fm = w.first_met, fa = w.first_amb, ft = w.first_tie;
        const bool decided = w.fixed_ok && (ft <= fm && ft <= fa || fm < fa);
        if (w.met0) {
            stop = 0;
        } else if (decided) {
            if (ft <= fm && ft <= fa && ft < np) bail = true;   // the walk meets the tie before any stop
            else stop = fm < np ? fm + 1 : np;
        } else {
            double acc = w.acc0;
            for (int p = 0; p < np && stop == np && !bail; p += 8) {
                uint32_t tq[8];
#pragma unroll
                for (int u = 0; u < 8; u++) tq[u] = p + u < np ? terms[p + u] : 0u;
                double sub[8], add[8];
#pragma unroll
                for (int u = 0; u < 8; u++) {
                    sub[u] = p + u < np ? ev[tq[u] & 0xffffu] : 0.0;
                    add[u] = p + u < np ? ev[tq[u] >> 16] : 0.0;
                }
                double a[8];
#pragma unroll
                for (int u = 0; u < 8; u++) {
                    acc -= sub[u];   // past np: - 0 + 0, never compared
                    acc += add[u];
                    a[u] = acc;
                }
#pragma unroll
                for (int u = 0; u < 8; u++) {
                    if (p + u >= np || stop < np || bail) continue;
                    if (w.tie[p + u]) bail = true;
                    else if (a[u] < tol) stop = p + u + 1;
                }
            }
        }
        w.fail = bail;
        w.stop = stop;
    }
    __syncthreads();
    if (w.fail) return false;
    // each level's new index: past its last popped entry
    if (tid < nl) w.nidx[tid] = w.start[tid];
    __syncthreads();
    for (int p = tid; p < w.stop; p += nth) {
        const int o = w.order[p], l = o >> 8, j = o & 255;
        atomicMax(&w.nidx[l], j + en[l * 64 + j]);
    }
    __syncthreads();
    if (tid < nl) {
        uint32_t r = w.rs[tid];
        for (int j = w.start[tid]; j < w.nidx[tid]; j++) r += sizes[(size_t)tid * B + j];
        rsz[tid] = r;
        index[tid] = (uint8_t)w.nidx[tid];
    }
    __syncthreads();
    return true;
}

// one CTA per field: all threads tabulate the efficiencies, warp 0 walks the
// levels (the exact heap walk on thread 0 when the warp walk declines)
template <class T>
__global__ void __launch_bounds__(256, 1) k_interpret(int nfields, int kind, int est_kind, const int* __restrict__ ndims,
                                                   const int* __restrict__ levels, double s, int B,
                                                   const uint32_t* __restrict__ sizes, uint64_t sz_stride,
                                                   const double* __restrict__ errs, uint64_t err_stride,
                                                   const double* __restrict__ tols, double tol0,
                                                   uint8_t* __restrict__ index, uint64_t idx_stride,
                                                   uint32_t* __restrict__ rsz, bool early) {
    // The kernel writes the plane counts that the previous retrieval's kernels
    // read, so it waits for them before the walk. With `early` (the host knows
    // that only this handle's reconstruction kernels, which write none of the
    // tables, ran since they were last written) the tables are read and
    // tabulated before that wait; otherwise everything waits.
    if (!early) {
        pdl_wait();
        pdl_release();
    }
    const int f = blockIdx.x;
    if (f >= nfields) return;
    const int L = levels[f];
    const int nl = L + 1;
    __shared__ uint32_t s_sizes[kMaxLevels * 64];
    __shared__ double s_errs[kMaxLevels * 65];
    __shared__ double s_ev[kMaxLevels * 65];
    __shared__ long long s_key[kMaxLevels * 64];
    __shared__ int8_t s_nan[kMaxLevels * 64];
    __shared__ int8_t s_en[kMaxLevels * 64];
    for (int i = threadIdx.x; i < nl * B; i += blockDim.x) s_sizes[i] = sizes[f * sz_stride + i];
    for (int i = threadIdx.x; i < nl * (B + 1); i += blockDim.x) s_errs[i] = errs[f * err_stride + i];
    __shared__ T s_tab[kMaxLevels];
    __shared__ uint8_t s_idx[kMaxLevels];
    uint8_t* gi = index + f * idx_stride;
    if (threadIdx.x < nl) s_idx[threadIdx.x] = gi[threadIdx.x];
    if ((est_kind == 2 || est_kind == 3) && threadIdx.x < nl && threadIdx.x < kMaxLevels)
        s_tab[threadIdx.x] = est_level_factor<T>(est_kind, ndims[f], L, s, threadIdx.x);
    __syncthreads();
    DevEstimator<T> est;
    est.init(est_kind, ndims[f], s_tab);
    for (int t = threadIdx.x; t < nl * (B + 1); t += blockDim.x) {
        const int l = t / (B + 1), j = t - l * (B + 1);
        s_ev[l * 65 + j] = (double)est.est((T)s_errs[t], l);
    }
    for (int t = threadIdx.x; t < nl * B; t += blockDim.x) {
        const int l = t / B, j = t - l * B;
        if (j < s_idx[l]) continue;    // planes already retrieved are never offered again
        double u;
        int num;
        eff_entry<T>(kind, est, B, s_sizes, s_errs, l, j, u, num);
        long long key;
        int nan;
        eff_key(u, key, nan);
        s_key[l * 64 + j] = key;
        s_nan[l * 64 + j] = (int8_t)nan;
        s_en[l * 64 + j] = (int8_t)num;
    }
    __syncthreads();
    if (early) {
        pdl_wait();
        pdl_release();
    }
    __shared__ uint32_t s_rs[kMaxLevels];
    __shared__ int s_ok;
    uint32_t* gr = rsz + f * idx_stride;
    const double tol = tols ? tols[f] : tol0;
    {   // the block-ordered walk; s_errs is free after the tabulation and holds its block keys
        __shared__ BlockWalkSmem s_bw;
        if (interpret_blocks(kind, nl, B, s_sizes, s_ev, s_key, s_nan, s_en, tol, s_idx, s_rs,
                             reinterpret_cast<long long*>(s_errs), s_bw)) {
            if (threadIdx.x < nl) {
                gi[threadIdx.x] = s_idx[threadIdx.x];
                gr[threadIdx.x] = s_rs[threadIdx.x];
            }
            return;
        }
    }
    if (threadIdx.x < 32) {
        const bool ok = nl <= 32 && interpret_warp(kind, nl, B, s_sizes, s_ev, s_key, s_nan, s_en, tol, s_idx, s_rs,
                                                   threadIdx.x);
        if (threadIdx.x == 0) s_ok = ok;
        __syncwarp();
        if (ok && threadIdx.x < nl) {
            gi[threadIdx.x] = s_idx[threadIdx.x];
            gr[threadIdx.x] = s_rs[threadIdx.x];
        }
    }
    __syncthreads();
    if (threadIdx.x == 0 && !s_ok) {
        uint8_t idx[kMaxLevels];
        uint32_t rs[kMaxLevels];
        for (int i = 0; i < nl; i++) idx[i] = gi[i];
        interpret_core(kind, nl, B, s_sizes, s_ev, s_key, s_nan, s_en, tol, idx, rs);
        for (int i = 0; i < nl; i++) { gi[i] = idx[i]; gr[i] = rs[i]; }
    }
}

}  // namespace

template <class T>
int launch_interpret(int nfields, int kind, int est_kind, const int* d_ndims, const int* d_levels, double s, int B,
                     const uint32_t* d_sizes, uint64_t sz_stride, const double* d_errs, uint64_t err_stride,
                     const double* d_tols, double tol0, uint8_t* d_index, uint64_t idx_stride, uint32_t* d_rsz,
                     cudaStream_t st, bool pdl, bool early) {
    count_launch();
    const cudaError_t e = launch_chain(pdl, k_interpret<T>, dim3(nfields), dim3(256), 0, st, nfields, kind, est_kind,
                                       d_ndims, d_levels, s, B, d_sizes, sz_stride, d_errs, err_stride, d_tols, tol0,
                                       d_index, idx_stride, d_rsz, pdl && early);
    if (e != cudaSuccess) return cuda_status(e, "k_interpret");
    return PRODM_OK;
}

template int launch_interpret<float>(int, int, int, const int*, const int*, double, int, const uint32_t*, uint64_t,
                                     const double*, uint64_t, const double*, double, uint8_t*, uint64_t,
                                     uint32_t*, cudaStream_t, bool, bool);
template int launch_interpret<double>(int, int, int, const int*, const int*, double, int, const uint32_t*, uint64_t,
                                      const double*, uint64_t, const double*, double, uint8_t*, uint64_t,
                                      uint32_t*, cudaStream_t, bool, bool);

}  // namespace prodm
