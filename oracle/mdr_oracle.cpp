// extern "C" surface of the CPU oracle (test infrastructure only; see
// mdr_oracle.hpp). Loaded by tests/ and bench.py's CPU baseline through ctypes.
#include "mdr_oracle.hpp"

using namespace mdr_oracle;

namespace {
std::vector<uint32_t> vec(const uint32_t* p, int n) { return std::vector<uint32_t>(p, p + n); }

template <class T>
size_t encode_any(int enc, const T* d, size_t n, int exp, int B, uint8_t* blob, uint32_t* sizes, double* errs) {
    using S = typename std::conditional<std::is_same<T, double>::value, uint64_t, uint32_t>::type;
    if (enc == 2) return pb_encode<T>(d, n, exp, B, blob, sizes);
    return enc == 0 ? nb_encode<T, S>(d, n, exp, B, blob, sizes, errs) : gr_encode<T, S>(d, n, exp, B, blob, sizes, errs);
}

// Composed refactor (ComposedRefactor.hpp:78-141): decompose, then per level
// interleave -> max -> frexp -> encode. Levels are written one after another
// into blob (each level = its plane streams in plane order).
template <class T>
int64_t refactor(const T* field, int ndims, const uint32_t* dims_, int L, int B, int enc, int hierarchical,
                 int collect, uint8_t* blob, uint32_t* sizes, T* bounds, double* errs, T* coeffs) {
    auto dims = vec(dims_, ndims);
    if (L > max_level(dims)) return -1;
    size_t N = 1; for (auto x : dims) N *= x;
    std::vector<T> data(field, field + N);
    decompose<T>(data.data(), dims, L, hierarchical != 0, {});
    if (coeffs) std::memcpy(coeffs, data.data(), N * sizeof(T));
    auto ld = level_dims(dims, L);
    auto le = level_elements(ld);
    std::vector<uint32_t> zero(ndims, 0);
    size_t off = 0;
    std::vector<T> buf;
    for (int i = 0; i <= L; i++) {
        buf.resize(le[i]);
        interleave<T>(data.data(), dims, ld[i], i == 0 ? zero : ld[i - 1], buf.data());
        T mx = max_abs(buf.data(), buf.size());
        bounds[i] = enc == 0 ? mx * 4 : mx;              // :111-112
        int e = 0; std::frexp(mx, &e);
        off += encode_any<T>(enc, buf.data(), buf.size(), e, B, blob + off, sizes + (size_t)i * B,
                             collect ? errs + (size_t)i * (B + 1) : nullptr);
    }
    return (int64_t)off;
}

template <class T>
void packed_recompose(const T* packed, const std::vector<uint32_t>& dims, int L, bool hier, T* out) {
    auto ld = level_dims(dims, L);
    auto le = level_elements(ld);
    std::vector<uint32_t> zero(dims.size(), 0);
    size_t N = 1; for (auto x : dims) N *= x;
    std::fill(out, out + N, (T)0);
    size_t off = 0;
    for (int l = 0; l <= L; l++) {
        reposition<T>(packed + off, dims, ld[l], l == 0 ? zero : ld[l - 1], out);
        off += le[l];
    }
    recompose<T>(out, dims, L, hier, {});
}

template <class T>
void packed_adjoint(const T* grad, const std::vector<uint32_t>& dims, int L, T* packed) {
    auto ld = level_dims(dims, L);
    auto le = level_elements(ld);
    std::vector<uint32_t> zero(dims.size(), 0);
    size_t N = 1; for (auto x : dims) N *= x;
    std::vector<T> g(grad, grad + N);
    recompose_adjoint<T>(g.data(), dims, L);
    size_t off = 0;
    for (int l = 0; l <= L; l++) {
        interleave<T>(g.data(), dims, ld[l], l == 0 ? zero : ld[l - 1], packed + off);
        off += le[l];
    }
}

// Retrieval that decodes all planes [0, index[l]) of every level and
// recomposes to full resolution (device-path semantics).
template <class T>
int retrieve_full(int ndims, const uint32_t* dims_, int L, int B, int enc, int hierarchical, const uint8_t* blob,
                  const uint32_t* sizes, const T* bounds, const uint8_t* index, T* out) {
    using S = typename std::conditional<std::is_same<T, double>::value, uint64_t, uint32_t>::type;
    auto dims = vec(dims_, ndims);
    size_t N = 1; for (auto x : dims) N *= x;
    auto ld = level_dims(dims, L);
    auto le = level_elements(ld);
    std::vector<uint32_t> zero(ndims, 0);
    std::fill(out, out + N, (T)0);
    size_t off = 0;
    GroupedState<S> st;
    PerBitState pst;
    std::vector<T> buf;
    for (int i = 0; i <= L; i++) {
        std::vector<const uint8_t*> planes(B);
        size_t o = off;
        for (int p = 0; p < B; p++) { planes[p] = blob + o; o += sizes[(size_t)i * B + p]; }
        int e = 0; std::frexp(enc == 0 ? bounds[i] / 4 : bounds[i], &e);
        buf.assign(le[i], 0);
        if (enc == 0) nb_decode<T, S>(planes.data(), le[i], e, 0, index[i], buf.data());
        else if (enc == 2) pb_decode<T>(pst, planes.data(), le[i], e, 0, index[i], i, buf.data());
        else if (gr_decode<T, S>(st, planes.data(), le[i], e, 0, index[i], i, buf.data()) != 0) return -2;
        reposition<T>(buf.data(), dims, ld[i], i == 0 ? zero : ld[i - 1], out);
        off = o;
    }
    recompose<T>(out, dims, L, hierarchical != 0, {});
    return 0;
}
}  // namespace

extern "C" {

int or_max_level(int ndims, const uint32_t* dims) { return max_level(vec(dims, ndims)); }

int or_adaptive_stopping(const uint32_t* raw, const uint32_t* comp, int B, int latter, uint8_t* compressed) {
    return adaptive_stopping(raw, comp, B, latter, compressed);
}
uint64_t or_zcb_size(const uint8_t* raw, uint64_t n) { return zcb_size(raw, n); }
uint64_t or_zcb_compress(const uint8_t* raw, uint64_t n, uint8_t* out) { return zcb_compress(raw, n, out); }
int64_t or_zcb_decompress(const uint8_t* in, uint64_t len, uint8_t* raw, uint64_t cap) {
    return zcb_decompress(in, len, raw, cap);
}

void or_level_dims(int ndims, const uint32_t* dims, int L, uint32_t* out) {
    auto ld = level_dims(vec(dims, ndims), L);
    for (int l = 0; l <= L; l++) for (int d = 0; d < ndims; d++) out[l * ndims + d] = ld[l][d];
}
void or_level_elements(int ndims, const uint32_t* dims, int L, uint32_t* out) {
    auto le = level_elements(level_dims(vec(dims, ndims), L));
    for (int l = 0; l <= L; l++) out[l] = le[l];
}

#define OR_T(SUF, T, S)                                                                                       \
    void or_interleave_##SUF(const T* data, int ndims, const uint32_t* dims, const uint32_t* fine,            \
                             const uint32_t* coarse, T* buf) {                                                \
        interleave<T>(data, vec(dims, ndims), vec(fine, ndims), vec(coarse, ndims), buf);                     \
    }                                                                                                         \
    void or_reposition_##SUF(const T* buf, int ndims, const uint32_t* dims, const uint32_t* fine,             \
                             const uint32_t* coarse, T* data) {                                               \
        reposition<T>(buf, vec(dims, ndims), vec(fine, ndims), vec(coarse, ndims), data);                     \
    }                                                                                                         \
    int64_t or_nb_encode_##SUF(const T* d, uint64_t n, int exp, int B, uint8_t* blob, uint32_t* sizes,       \
                               double* errs) {                                                                \
        return (int64_t)nb_encode<T, S>(d, n, exp, B, blob, sizes, errs);                                     \
    }                                                                                                         \
    int64_t or_gr_encode_##SUF(const T* d, uint64_t n, int exp, int B, uint8_t* blob, uint32_t* sizes,       \
                               double* errs) {                                                                \
        return (int64_t)gr_encode<T, S>(d, n, exp, B, blob, sizes, errs);                                     \
    }                                                                                                         \
    int or_nb_decode_##SUF(const uint8_t* blob, const uint32_t* sizes, uint64_t n, int exp, int s, int num,   \
                           T* out) {                                                                          \
        std::vector<const uint8_t*> planes(num > 0 ? num : 1);                                                \
        size_t o = 0;                                                                                         \
        for (int i = 0; i < num; i++) { planes[i] = blob + o; o += sizes[i]; }                                \
        nb_decode<T, S>(planes.data(), n, exp, s, num, out);                                                  \
        return 0;                                                                                             \
    }                                                                                                         \
    int64_t or_pb_encode_##SUF(const T* d, uint64_t n, int exp, int B, uint8_t* blob, uint32_t* sizes) {      \
        return (int64_t)pb_encode<T>(d, n, exp, B, blob, sizes);                                              \
    }                                                                                                         \
    void* or_pb_state_new_##SUF() { return new PerBitState(); }                                               \
    void or_pb_state_free_##SUF(void* p) { delete (PerBitState*)p; }                                          \
    int or_pb_decode_##SUF(void* st, const uint8_t* blob, const uint32_t* sizes, uint64_t n, int exp, int s,  \
                           int num, int level, T* out) {                                                      \
        std::vector<const uint8_t*> planes(num > 0 ? num : 1);                                                \
        size_t o = 0;                                                                                         \
        for (int i = 0; i < num; i++) { planes[i] = blob + o; o += sizes[i]; }                                \
        pb_decode<T>(*(PerBitState*)st, planes.data(), n, exp, s, num, level, out);                           \
        return 0;                                                                                             \
    }                                                                                                         \
    void* or_gr_state_new_##SUF() { return new GroupedState<S>(); }                                           \
    void or_gr_state_free_##SUF(void* p) { delete (GroupedState<S>*)p; }                                      \
    int or_gr_decode_##SUF(void* st, const uint8_t* blob, const uint32_t* sizes, uint64_t n, int exp, int s,  \
                           int num, int level, T* out) {                                                      \
        std::vector<const uint8_t*> planes(num > 0 ? num : 1);                                                \
        size_t o = 0;                                                                                         \
        for (int i = 0; i < num; i++) { planes[i] = blob + o; o += sizes[i]; }                                \
        return gr_decode<T, S>(*(GroupedState<S>*)st, planes.data(), n, exp, s, num, level, out);             \
    }                                                                                                         \
    void or_max_collect_##SUF(T bound, int B, double* out) { max_collect<T>(bound, B, out); }                 \
    void or_sq_collect_##SUF(const T* d, uint64_t n, int B, T mx, double* out) { sq_collect<T>(d, n, B, mx, out); } \
    T or_max_abs_##SUF(const T* d, uint64_t n) { return max_abs<T>(d, n); }                                   \
    void or_decompose_##SUF(T* d, int ndims, const uint32_t* dims, int L, int hier) {                         \
        decompose<T>(d, vec(dims, ndims), L, hier != 0, {});                                                  \
    }                                                                                                         \
    void or_recompose_##SUF(T* d, int ndims, const uint32_t* dims, int L, int hier) {                         \
        recompose<T>(d, vec(dims, ndims), L, hier != 0, {});                                                  \
    }                                                                                                         \
    void or_recompose_strided_##SUF(T* d, int ndims, const uint32_t* dims, int L, int hier,                   \
                                    const uint32_t* strides) {                                                \
        recompose<T>(d, vec(dims, ndims), L, hier != 0, vec(strides, ndims));                                 \
    }                                                                                                         \
    /* packed levels (level 0 box, then box(l) minus box(l-1) per level, in     \
       interleaved order) -> natural field, and its transpose (hierarchical) */ \
    void or_recompose_packed_##SUF(const T* packed, int ndims, const uint32_t* dims, int L, int hier, T* out) { \
        packed_recompose<T>(packed, vec(dims, ndims), L, hier != 0, out);                                     \
    }                                                                                                         \
    void or_recompose_adjoint_##SUF(const T* grad, int ndims, const uint32_t* dims, int L, T* packed) {      \
        packed_adjoint<T>(grad, vec(dims, ndims), L, packed);                                                 \
    }                                                                                                         \
    int64_t or_refactor_##SUF(const T* f, int ndims, const uint32_t* dims, int L, int B, int enc, int hier,   \
                              int collect, uint8_t* blob, uint32_t* sizes, T* bounds, double* errs,           \
                              T* coeffs) {                                                                    \
        return refactor<T>(f, ndims, dims, L, B, enc, hier, collect, blob, sizes, bounds, errs, coeffs);      \
    }                                                                                                         \
    int or_retrieve_##SUF(int ndims, const uint32_t* dims, int L, int B, int enc, int hier,                   \
                          const uint8_t* blob, const uint32_t* sizes, const T* bounds, const uint8_t* index,  \
                          T* out) {                                                                           \
        return retrieve_full<T>(ndims, dims, L, B, enc, hier, blob, sizes, bounds, index, out);               \
    }                                                                                                         \
    void or_interpret_##SUF(int kind, int est_kind, int ndims, int L, double s, int nl, int B,                \
                            const uint32_t* sizes, const double* errs, double tol, uint8_t* index,            \
                            uint32_t* rsz) {                                                                  \
        Estimator<T> est(est_kind, ndims, L, s);                                                              \
        interpret<T>(kind, est, nl, B, sizes, errs, tol, index, rsz);                                         \
    }

OR_T(f32, float, uint32_t)
OR_T(f64, double, uint64_t)

void or_qoi_values_f64(const double* vx, const double* vy, const double* vz, const double* p, const double* d,
                       uint64_t n, double* vtot, double* temp, double* c, double* mach, double* pt, double* mu) {
    qoi_values(vx, vy, vz, p, d, (size_t)n, vtot, temp, c, mach, pt, mu);
}
void or_qoi_vtot_bound_f64(const double* vx, const double* vy, const double* vz, uint64_t n, double ebx, double eby,
                           double ebz, double* out) {
    vtot_bound(vx, vy, vz, (size_t)n, ebx, eby, ebz, out);
}
void or_qoi_t_bound_f64(const double* p, const double* d, uint64_t n, double ebp, double ebd, double* out) {
    t_bound(p, d, (size_t)n, ebp, ebd, out);
}

}  // extern "C"
