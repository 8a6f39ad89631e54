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
#include "common.cuh"
#include "kernels.cuh"

namespace prodm {

namespace {

constexpr int kMaxLevels = 17;

template <class T>
struct DevEstimator {
    int kind;
    T c;
    T table[kMaxLevels];
    __device__ void init(int k, int ndims, int L, double s) {
        kind = k;
        c = 0;
        if (k == 1) {
            double cc = ndims == 1 ? 1.0 + sqrt(3.0) / 2 : ndims == 2 ? 1.0 + 9.0 / 4 : 1.0 + 21.0 * sqrt(3.0) / 8;
            c = (T)cc;
            c *= 4;
        } else if (k == 2) {
            for (int i = 0; i <= L && i < kMaxLevels; i++) table[i] = (T)exp2((double)(ndims * (L - i)));
        } else if (k == 3) {
            T sT = (T)s;
            for (int i = 0; i <= L && i < kMaxLevels; i++) table[i] = (T)exp2((double)(2 * sT * i + ndims * (L - i)));
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

struct Item { double u; int level; int num; };

struct DevHeap {
    Item h[kMaxLevels + 1];
    int len;
    __device__ static bool less(const Item& a, const Item& b) { return a.u < b.u; }
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

template <class T>
__device__ void interpret_core(int kind, const DevEstimator<T>& est, int nl, int B, const uint32_t* __restrict__ sizes,
                               const double* __restrict__ errs, double tol, uint8_t* index, uint32_t* rsz) {
    auto E = [&](int l, int j) { return errs[(size_t)l * (B + 1) + j]; };
    auto S = [&](int l, int j) { return sizes[(size_t)l * B + j]; };
    for (int i = 0; i < nl; i++) rsz[i] = 0;
    double acc = 0;
    for (int i = 0; i < nl; i++) acc += est.est((T)E(i, index[i]), i);
    DevHeap heap;
    heap.len = 0;
    if (kind == 0) {
        for (int i = 0; i < nl; i++) {
            double g = est.gain((T)E(i, index[i]), (T)E(i, index[i] + 1), i);
            heap.push({g / S(i, index[i]), i, 1});
        }
        bool met = false;
        while (!met && heap.len > 0) {
            Item t = heap.h[0];
            heap.pop();
            int i = t.level, j = index[i];
            rsz[i] += S(i, j);
            acc -= est.est((T)E(i, j), i);
            acc += est.est((T)E(i, j + 1), i);
            if (acc < tol) met = true;
            index[i]++;
            if (index[i] != B) {
                double g = est.gain((T)E(i, index[i]), (T)E(i, index[i] + 1), i);
                heap.push({g / S(i, index[i]), i, 1});
            }
        }
        return;
    }
    if (kind == 1) {
        if (acc < tol) return;
        double minerr = acc;
        for (int i = 0; i < nl; i++) {
            minerr -= est.est((T)E(i, index[i]), i);
            minerr += est.est((T)E(i, B), i);
            if (index[i] == 0) {
                rsz[i] += S(i, 0);
                acc -= est.est((T)E(i, 0), i);
                acc += est.est((T)E(i, 1), i);
                index[i]++;
            }
            if (index[i] != B) {
                double g = est.gain((T)E(i, index[i]), (T)E(i, index[i] + 1), i);
                heap.push({g / S(i, index[i]), i, 1});
            }
            if (minerr < tol) break;
        }
        bool met = acc < tol;
        while (!met && heap.len > 0) {
            Item t = heap.h[0];
            heap.pop();
            int i = t.level, j = index[i];
            rsz[i] += S(i, j);
            acc -= est.est((T)E(i, j), i);
            acc += est.est((T)E(i, j + 1), i);
            if (acc < tol) met = true;
            index[i]++;
            if (index[i] != B) {
                double g = est.gain((T)E(i, index[i]), (T)E(i, index[i] + 1), i);
                heap.push({g / S(i, index[i]), i, 1});
            }
        }
        return;
    }
    // estimated_efficiency (GreedyBasedSizeInterpreter.hpp:228-248), warp-parallel:
    // candidate i (run of i planes) has efficiency gain(E[idx], E[idx+i]) /
    // (sizes[idx] + ... + sizes[idx+i-1]) with the reference's u32 size sums;
    // the sequential loop stops at the first i >= 2 whose predecessor is
    // positive and larger, which a ballot finds directly.
    const int lane = threadIdx.x & 31;
    auto eff = [&](int idx, int l) {
        const int cnt = B - idx - 1;             // largest candidate run the loop visits
        uint32_t carry = 0;
        double prev_last = 0.0;
        int cn = -1;
        double ce = 0.0;
        for (int base = 0; base <= (cnt > 1 ? cnt : 1); base += 32) {
            const int i = base + lane;
            uint32_t sz = (i >= 1 && idx + i - 1 < B) ? S(l, idx + i - 1) : 0u;
            uint32_t incl = sz;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= o) incl += t;
            }
            const uint32_t ns = carry + incl;
            double ne = 0.0;
            if (i >= 1 && idx + i <= B) ne = (double)est.gain((T)E(l, idx), (T)E(l, idx + i), l) / ns;
            double prev = __shfl_up_sync(0xffffffffu, ne, 1);
            if (lane == 0) prev = prev_last;
            const bool stop = i >= 2 && i <= cnt && (prev > 0) && (prev > ne);
            const unsigned m = __ballot_sync(0xffffffffu, stop);
            if (m) {
                const int bi = base + __ffs(m) - 1;      // first stopping candidate
                cn = bi - 1;
                const int src = cn - base;
                const double a = __shfl_sync(0xffffffffu, ne, src < 0 ? 0 : src);
                ce = src < 0 ? prev_last : a;
                break;
            }
            prev_last = __shfl_sync(0xffffffffu, ne, 31);
            carry = __shfl_sync(0xffffffffu, ns, 31);
        }
        if (cn < 0) {
            cn = cnt >= 2 ? cnt : 1;
            // efficiency of the accepted run cn (recomputed, same expression)
            uint32_t tot = 0;
            for (int j = 0; j < cn; j++) tot += S(l, idx + j);
            ce = (double)est.gain((T)E(l, idx), (T)E(l, idx + cn), l) / tot;
        }
        return Item{ce, l, cn};
    };
    for (int i = 0; i < nl; i++)
        if (index[i] != B) heap.push(eff(index[i], i));
    bool met = acc < tol;
    if (met) return;
    while (!met && heap.len > 0) {
        Item t = heap.h[0];
        heap.pop();
        int i = t.level, j = index[i], num = t.num;
        for (int k = 0; k < num; k++) rsz[i] += S(i, j + k);
        acc -= est.est((T)E(i, j), i);
        acc += est.est((T)E(i, j + num), i);
        if (acc < tol) met = true;
        index[i] += num;
        if (index[i] != B) heap.push(eff(index[i], i));
    }
}

// all lanes of the warp run the same sequence on private copies; lane 0 stores
template <class T>
__device__ void interpret_one(int kind, const DevEstimator<T>& est, int nl, int B, const uint32_t* __restrict__ sizes,
                              const double* __restrict__ errs, double tol, uint8_t* __restrict__ index_io,
                              uint32_t* __restrict__ rsz_io) {
    uint8_t index[kMaxLevels];
    uint32_t rsz[kMaxLevels];
    for (int i = 0; i < nl; i++) index[i] = index_io[i];
    interpret_core<T>(kind, est, nl, B, sizes, errs, tol, index, rsz);
    __syncwarp();
    if ((threadIdx.x & 31) == 0)
        for (int i = 0; i < nl; i++) { index_io[i] = index[i]; rsz_io[i] = rsz[i]; }
}

// one thread per field: field f uses sizes + f*sz_stride etc.
template <class T>
__global__ void k_interpret(int nfields, int kind, int est_kind, const int* __restrict__ ndims,
                            const int* __restrict__ levels, double s, int B, const uint32_t* __restrict__ sizes,
                            uint64_t sz_stride, const double* __restrict__ errs, uint64_t err_stride,
                            const double* __restrict__ tols, double tol0, uint8_t* __restrict__ index,
                            uint64_t idx_stride, uint32_t* __restrict__ rsz) {
    const int f = blockIdx.x;              // one warp per field; all lanes run the same steps
    if (f >= nfields) return;
    int L = levels[f];
    DevEstimator<T> est;
    est.init(est_kind, ndims[f], L, s);
    // stage this field's size and error tables in shared memory (latency)
    __shared__ uint32_t s_sizes[kMaxLevels * 64];
    __shared__ double s_errs[kMaxLevels * 65];
    const int nl = L + 1;
    for (int i = threadIdx.x; i < nl * B; i += blockDim.x) s_sizes[i] = sizes[f * sz_stride + i];
    for (int i = threadIdx.x; i < nl * (B + 1); i += blockDim.x) s_errs[i] = errs[f * err_stride + i];
    __syncwarp();
    interpret_one<T>(kind, est, L + 1, B, s_sizes, s_errs, tols ? tols[f] : tol0, index + f * idx_stride,
                     rsz + f * idx_stride);
}

}  // namespace

template <class T>
int launch_interpret(int nfields, int kind, int est_kind, const int* d_ndims, const int* d_levels, double s, int B,
                     const uint32_t* d_sizes, uint64_t sz_stride, const double* d_errs, uint64_t err_stride,
                     const double* d_tols, double tol0, uint8_t* d_index, uint64_t idx_stride, uint32_t* d_rsz,
                     cudaStream_t st) {
    k_interpret<T><<<nfields, 32, 0, st>>>(nfields, kind, est_kind, d_ndims, d_levels, s, B, d_sizes,
                                                           sz_stride, d_errs, err_stride, d_tols, tol0, d_index,
                                                           idx_stride, d_rsz);
    PRODM_CHECK_LAUNCH("k_interpret");
    return PRODM_OK;
}

template int launch_interpret<float>(int, int, int, const int*, const int*, double, int, const uint32_t*, uint64_t,
                                     const double*, uint64_t, const double*, double, uint8_t*, uint64_t,
                                     uint32_t*, cudaStream_t);
template int launch_interpret<double>(int, int, int, const int*, const int*, double, int, const uint32_t*, uint64_t,
                                      const double*, uint64_t, const double*, double, uint8_t*, uint64_t,
                                      uint32_t*, cudaStream_t);

}  // namespace prodm
