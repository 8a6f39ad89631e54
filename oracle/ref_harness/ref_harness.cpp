// Reference harness (test infrastructure only): compiles lxAltria/ProDM's own
// MDR headers, unmodified, from the reference tree and exposes their
// components through extern "C" entry points so that the oracle restatement
// and the golden vectors can be checked against the reference itself.
// The MGARDx decomposer the reference includes is absent; shim/ forwards it to
// the oracle's restatement, so composed-refactor parity at that boundary stays
// unpinned. Built into oracle/_ref/ by oracle/build_oracle.py.
#include <iostream>
#include <mutex>
#include <sstream>
#include <vector>
#include <string>
#include <cstring>
#include <cstdint>
#include <cmath>
#include <queue>
#include <cassert>
#include <type_traits>
#include "MDR/RefactorUtils.hpp"
#include "MDR/Interleaver/Interleaver.hpp"
#include "MDR/BitplaneEncoder/BitplaneEncoder.hpp"
#include "MDR/ErrorCollector/ErrorCollector.hpp"
#include "MDR/ErrorEstimator/ErrorEstimator.hpp"
#include "MDR/SizeInterpreter/SizeInterpreter.hpp"
#include "MDR/Refactor/Refactor.hpp"
#include "MDR/LosslessCompressor/AdaptiveLevelCompressor.hpp"
#include "MDR/Reconstructor/Reconstructor.hpp"
#include "qoi_utils.hpp"

namespace {
// The reference's classes print to std::cout. While any harness call runs,
// std::cout writes into one stateless discarding buffer; the first caller
// swaps it in and the last one restores the original, so calls from several
// threads at once (the benchmark's CPU arm) never leave std::cout pointing at
// a buffer that is gone.
struct DiscardBuf : std::streambuf {
    int overflow(int c) override { return c == EOF ? 0 : c; }
    std::streamsize xsputn(const char*, std::streamsize n) override { return n; }
};
struct Quiet {
    static std::mutex& mu() { static std::mutex m; return m; }
    static int& depth() { static int d = 0; return d; }
    static std::streambuf*& saved() { static std::streambuf* s = nullptr; return s; }
    static DiscardBuf& sink() { static DiscardBuf b; return b; }
    Quiet() {
        std::lock_guard<std::mutex> lock(mu());
        if (depth()++ == 0) saved() = std::cout.rdbuf(&sink());
    }
    ~Quiet() {
        std::lock_guard<std::mutex> lock(mu());
        if (--depth() == 0) std::cout.rdbuf(saved());
    }
};
std::vector<uint32_t> vec(const uint32_t* p, int n) { return std::vector<uint32_t>(p, p + n); }

template <class T, class S, class Enc>
int64_t enc_call(const T* d, uint64_t n, int exp, int B, uint8_t* blob, uint32_t* sizes, double* errs) {
    Enc enc;
    std::vector<uint32_t> ss;
    std::vector<uint8_t*> st;
    if (errs) {
        std::vector<double> e;
        st = enc.encode(d, (int32_t)n, exp, (uint8_t)B, ss, e);
        for (int i = 0; i <= B; i++) errs[i] = e[i];
    } else {
        st = enc.encode(d, (int32_t)n, exp, (uint8_t)B, ss);
    }
    size_t off = 0;
    for (int p = 0; p < B; p++) {
        sizes[p] = ss[p];
        std::memcpy(blob + off, st[p], ss[p]);
        off += ss[p];
        free(st[p]);
    }
    return (int64_t)off;
}

template <class T, class Est>
void interp_call(int kind, const Est& est, int nl, int B, const uint32_t* sizes, const double* errs, double tol,
                 uint8_t* index, uint32_t* rsz) {
    std::vector<std::vector<uint32_t>> ls(nl);
    std::vector<std::vector<double>> le(nl);
    for (int l = 0; l < nl; l++) {
        ls[l].assign(sizes + (size_t)l * B, sizes + (size_t)(l + 1) * B);
        le[l].assign(errs + (size_t)l * (B + 1), errs + (size_t)(l + 1) * (B + 1));
    }
    std::vector<uint8_t> idx(index, index + nl);
    std::vector<uint32_t> r;
    Quiet q;
    if (kind == 0) r = MDR::GreedyBasedSizeInterpreter<Est>(est).interpret_retrieve_size(ls, le, tol, idx);
    else if (kind == 1) r = MDR::SignExcludeGreedyBasedSizeInterpreter<Est>(est).interpret_retrieve_size(ls, le, tol, idx);
    else r = MDR::NegaBinaryGreedyBasedSizeInterpreter<Est>(est).interpret_retrieve_size(ls, le, tol, idx);
    for (int l = 0; l < nl; l++) { index[l] = idx[l]; rsz[l] = r[l]; }
}

template <class T>
void interp_any(int kind, int est_kind, int ndims, int L, double s, int nl, int B, const uint32_t* sizes,
                const double* errs, double tol, uint8_t* index, uint32_t* rsz) {
    switch (est_kind) {
        case 0: interp_call<T>(kind, MDR::MaxErrorEstimatorHB<T>(), nl, B, sizes, errs, tol, index, rsz); break;
        case 1: interp_call<T>(kind, MDR::MaxErrorEstimatorOB<T>(ndims), nl, B, sizes, errs, tol, index, rsz); break;
        case 2: interp_call<T>(kind, MDR::L2ErrorEstimator_HB<T>(ndims, L), nl, B, sizes, errs, tol, index, rsz); break;
        default: interp_call<T>(kind, MDR::SNormErrorEstimator<T>(ndims, L, (T)s), nl, B, sizes, errs, tol, index, rsz); break;
    }
}

// ComposedRefactor + ComposedReconstructor driven as test/test_mdr_refactor.cpp
// and test/test_mdr_reconstructor.cpp do, on files under dir (level
// compressor Comp: NullLevelCompressor, or AdaptiveLevelCompressor(latter)).
template <class T, class S, class Dec, class Enc, class Est, class Comp = MDR::NullLevelCompressor>
int composed_roundtrip(const T* field, int ndims, const uint32_t* dims, int L, int B, bool negabinary,
                       const char* dir, int ntol, const double* tols, T* outs, uint64_t* retrieved,
                       const Comp& comp = Comp()) {
    std::string d(dir);
    std::string meta = d + "/metadata.bin";
    std::vector<std::string> files;
    for (int i = 0; i <= L; i++) files.push_back(d + "/level_" + std::to_string(i) + ".bin");
    size_t N = 1; for (int i = 0; i < ndims; i++) N *= dims[i];
    Quiet q;
    {
        auto refactor = MDR::ComposedRefactor<T, Dec, MDR::DirectInterleaver<T>, Enc, Comp,
                                              MDR::MaxErrorCollector<T>, MDR::ConcatLevelFileWriter>(
            Dec(), MDR::DirectInterleaver<T>(), Enc(), comp, MDR::MaxErrorCollector<T>(),
            MDR::ConcatLevelFileWriter(meta, files));
        refactor.negabinary = negabinary;
        refactor.refactor(field, vec(dims, ndims), (uint8_t)L, (uint8_t)B);
    }
    auto rec = MDR::ComposedReconstructor<T, Dec, MDR::DirectInterleaver<T>, Enc, Comp,
                                          MDR::SignExcludeGreedyBasedSizeInterpreter<Est>, Est,
                                          MDR::ConcatLevelFileRetriever>(
        Dec(), MDR::DirectInterleaver<T>(), Enc(), comp,
        MDR::SignExcludeGreedyBasedSizeInterpreter<Est>(Est()), MDR::ConcatLevelFileRetriever(meta, files));
    rec.load_metadata();
    for (int t = 0; t < ntol; t++) {
        T* r = rec.progressive_reconstruct(tols[t], -1);
        if (!r) return -1;
        std::memcpy(outs + (size_t)t * N, r, N * sizeof(T));
        retrieved[t] = rec.get_retrieved_size();
    }
    return 0;
}
}  // namespace

extern "C" {

#define REF_T(SUF, T, S)                                                                                        \
    int64_t ref_nb_encode_##SUF(const T* d, uint64_t n, int exp, int B, uint8_t* blob, uint32_t* sizes,        \
                                double* errs) {                                                                 \
        return enc_call<T, S, MDR::NegaBinaryBPEncoder<T, S>>(d, n, exp, B, blob, sizes, errs);                 \
    }                                                                                                           \
    int64_t ref_gr_encode_##SUF(const T* d, uint64_t n, int exp, int B, uint8_t* blob, uint32_t* sizes,        \
                                double* errs) {                                                                 \
        return enc_call<T, S, MDR::GroupedBPEncoder<T, S>>(d, n, exp, B, blob, sizes, errs);                    \
    }                                                                                                           \
    void* ref_nb_new_##SUF() { return new MDR::NegaBinaryBPEncoder<T, S>(); }                                   \
    void ref_nb_free_##SUF(void* p) { delete (MDR::NegaBinaryBPEncoder<T, S>*)p; }                              \
    void* ref_gr_new_##SUF() { return new MDR::GroupedBPEncoder<T, S>(); }                                      \
    void ref_gr_free_##SUF(void* p) { delete (MDR::GroupedBPEncoder<T, S>*)p; }                                 \
    int ref_decode_##SUF(void* h, int grouped, const uint8_t* blob, const uint32_t* sizes, uint64_t n, int exp, \
                         int s, int num, int level, T* out) {                                                   \
        std::vector<const uint8_t*> planes;                                                                     \
        size_t o = 0;                                                                                           \
        for (int i = 0; i < num; i++) { planes.push_back(blob + o); o += sizes[i]; }                            \
        T* r = grouped ? ((MDR::GroupedBPEncoder<T, S>*)h)->progressive_decode(planes, (int32_t)n, exp,        \
                                                                                (uint8_t)s, (uint8_t)num, level) \
                       : ((MDR::NegaBinaryBPEncoder<T, S>*)h)->progressive_decode(planes, (int32_t)n, exp,     \
                                                                                   (uint8_t)s, (uint8_t)num,    \
                                                                                   level);                      \
        std::memcpy(out, r, n * sizeof(T));                                                                     \
        free(r);                                                                                                \
        return 0;                                                                                               \
    }                                                                                                           \
    void ref_max_collect_##SUF(T bound, int B, double* out) {                                                   \
        auto v = MDR::MaxErrorCollector<T>().collect_level_error(nullptr, 0, B, bound);                         \
        for (int i = 0; i <= B; i++) out[i] = v[i];                                                             \
    }                                                                                                           \
    void ref_sq_collect_##SUF(const T* d, uint64_t n, int B, T mx, double* out) {                               \
        auto v = MDR::SquaredErrorCollector<T>().collect_level_error(d, n, B, mx);                              \
        for (int i = 0; i <= B; i++) out[i] = v[i];                                                             \
    }                                                                                                           \
    void ref_interleave_##SUF(const T* data, int ndims, const uint32_t* dims, const uint32_t* fine,             \
                              const uint32_t* coarse, T* buf) {                                                 \
        MDR::DirectInterleaver<T>().interleave(data, vec(dims, ndims), vec(fine, ndims), vec(coarse, ndims),   \
                                                buf);                                                           \
    }                                                                                                           \
    void ref_reposition_##SUF(const T* buf, int ndims, const uint32_t* dims, const uint32_t* fine,             \
                              const uint32_t* coarse, T* data) {                                                \
        MDR::DirectInterleaver<T>().reposition(buf, vec(dims, ndims), vec(fine, ndims), vec(coarse, ndims),    \
                                                data);                                                          \
    }                                                                                                           \
    void ref_interpret_##SUF(int kind, int est_kind, int ndims, int L, double s, int nl, int B,                 \
                             const uint32_t* sizes, const double* errs, double tol, uint8_t* index,             \
                             uint32_t* rsz) {                                                                   \
        interp_any<T>(kind, est_kind, ndims, L, s, nl, B, sizes, errs, tol, index, rsz);                        \
    }                                                                                                           \
    void ref_level_dims_##SUF(int ndims, const uint32_t* dims, int L, uint32_t* out, uint32_t* elems) {         \
        auto ld = MDR::compute_level_dims(vec(dims, ndims), L);                                                 \
        auto le = MDR::compute_level_elements(ld, L);                                                           \
        for (int l = 0; l <= L; l++) {                                                                          \
            for (int d = 0; d < ndims; d++) out[l * ndims + d] = ld[l][d];                                      \
            elems[l] = le[l];                                                                                   \
        }                                                                                                       \
    }                                                                                                           \
    int ref_composed_##SUF(const T* field, int ndims, const uint32_t* dims, int L, int B, int enc, int hier,    \
                           const char* dir, int ntol, const double* tols, T* outs, uint64_t* retrieved) {       \
        if (hier) {                                                                                             \
            if (enc == 0)                                                                                       \
                return composed_roundtrip<T, S, MDR::MGARDHierarchicalDecomposer<T>,                            \
                                          MDR::NegaBinaryBPEncoder<T, S>, MDR::MaxErrorEstimatorHB<T>>(         \
                    field, ndims, dims, L, B, true, dir, ntol, tols, outs, retrieved);                          \
            return composed_roundtrip<T, S, MDR::MGARDHierarchicalDecomposer<T>, MDR::GroupedBPEncoder<T, S>,   \
                                      MDR::MaxErrorEstimatorHB<T>>(field, ndims, dims, L, B, false, dir, ntol,  \
                                                                   tols, outs, retrieved);                      \
        }                                                                                                       \
        if (enc == 0)                                                                                           \
            return composed_roundtrip<T, S, MDR::MGARDOrthoganalDecomposer<T>, MDR::NegaBinaryBPEncoder<T, S>,  \
                                      MDR::MaxErrorEstimatorOB<T>>(field, ndims, dims, L, B, true, dir, ntol,   \
                                                                   tols, outs, retrieved);                      \
        return composed_roundtrip<T, S, MDR::MGARDOrthoganalDecomposer<T>, MDR::GroupedBPEncoder<T, S>,         \
                                  MDR::MaxErrorEstimatorOB<T>>(field, ndims, dims, L, B, false, dir, ntol,      \
                                                               tols, outs, retrieved);                          \
    }

REF_T(f32, float, uint32_t)
REF_T(f64, double, uint64_t)

// The same round trip with the reference's zstd stage,
// AdaptiveLevelCompressor(latter) (hierarchical basis; enc 0 negabinary,
// else grouped): the level files and metadata a stock refactor writes.
extern "C" int ref_composed_zstd_f32(const float* field, int ndims, const uint32_t* dims, int L, int B, int enc,
                                     int latter, const char* dir, int ntol, const double* tols, float* outs,
                                     uint64_t* retrieved) {
    const MDR::AdaptiveLevelCompressor comp(latter);
    if (enc == 0)
        return composed_roundtrip<float, uint32_t, MDR::MGARDHierarchicalDecomposer<float>,
                                  MDR::NegaBinaryBPEncoder<float, uint32_t>, MDR::MaxErrorEstimatorHB<float>,
                                  MDR::AdaptiveLevelCompressor>(field, ndims, dims, L, B, true, dir, ntol, tols, outs,
                                                                retrieved, comp);
    return composed_roundtrip<float, uint32_t, MDR::MGARDHierarchicalDecomposer<float>,
                              MDR::GroupedBPEncoder<float, uint32_t>, MDR::MaxErrorEstimatorHB<float>,
                              MDR::AdaptiveLevelCompressor>(field, ndims, dims, L, B, false, dir, ntol, tols, outs,
                                                            retrieved, comp);
}

// PerBitBPEncoder with the stream word type the GE applications instantiate it
// with (refactorGE.cpp:72: PerBitBPEncoder<Type, uint32_t>)
#define REF_PB(SUF, T)                                                                                          \
    int64_t ref_pb_encode_##SUF(const T* d, uint64_t n, int exp, int B, uint8_t* blob, uint32_t* sizes) {      \
        return enc_call<T, uint32_t, MDR::PerBitBPEncoder<T, uint32_t>>(d, n, exp, B, blob, sizes, nullptr);    \
    }                                                                                                           \
    void* ref_pb_new_##SUF() { return new MDR::PerBitBPEncoder<T, uint32_t>(); }                                \
    void ref_pb_free_##SUF(void* p) { delete (MDR::PerBitBPEncoder<T, uint32_t>*)p; }                           \
    int ref_pb_decode_##SUF(void* h, const uint8_t* blob, const uint32_t* sizes, uint64_t n, int exp, int s,    \
                            int num, int level, T* out) {                                                       \
        std::vector<const uint8_t*> planes;                                                                     \
        size_t o = 0;                                                                                           \
        for (int i = 0; i < num; i++) { planes.push_back(blob + o); o += sizes[i]; }                            \
        T* r = ((MDR::PerBitBPEncoder<T, uint32_t>*)h)->progressive_decode(planes, (int32_t)n, exp, (uint8_t)s, \
                                                                          (uint8_t)num, level);                 \
        std::memcpy(out, r, n * sizeof(T));                                                                     \
        free(r);                                                                                                \
        return 0;                                                                                               \
    }                                                                                                           \
    int ref_composed_pb_##SUF(const T* field, int ndims, const uint32_t* dims, int L, int B, const char* dir,   \
                              int ntol, const double* tols, T* outs, uint64_t* retrieved) {                     \
        return composed_roundtrip<T, uint32_t, MDR::MGARDHierarchicalDecomposer<T>,                             \
                                  MDR::PerBitBPEncoder<T, uint32_t>, MDR::MaxErrorEstimatorHB<T>>(              \
            field, ndims, dims, L, B, false, dir, ntol, tols, outs, retrieved);                                 \
    }

REF_PB(f32, float)
REF_PB(f64, double)

// One step of the benchmark workload on the reference's own classes: the
// refactor loop of ComposedRefactor::refactor (ComposedRefactor.hpp:78-141:
// decompose, then per level interleave, level max, exponent, encode) and, per
// tolerance, the progressive loop of ComposedReconstructor::reconstruct
// (ComposedReconstructor.hpp:27-100, :187-258: interpret, decode the new
// planes of each level, reposition, recompose, add the previous
// reconstruction). The squared-error tables come from the encoder's
// error-collecting overload (NegaBinaryBPEncoder.hpp:65-125), the call
// ComposedRefactor leaves commented out (:117-118), because its reconstructor
// needs them for an L2 tolerance; streams stay in memory (NullLevelCompressor,
// no files). tols are absolute squared tolerances. Returns the step's
// algorithmic bytes (field read + all streams written; per tolerance the
// streams retrieved so far + the field written), or -1.
extern "C" int64_t ref_headline_step_f32(const float* field, const uint32_t* dims3, int L, int B, int ntol,
                                         const double* tols, float* out) {
    using Enc = MDR::NegaBinaryBPEncoder<float, uint32_t>;
    std::vector<uint32_t> dims(dims3, dims3 + 3);
    const size_t N = (size_t)dims[0] * dims[1] * dims[2];
    std::vector<float> data(field, field + N);
    MDR::MGARDHierarchicalDecomposer<float> decomposer;
    MDR::DirectInterleaver<float> interleaver;
    Enc encoder;
    Quiet q;
    decomposer.decompose(data.data(), dims, (uint32_t)L);
    auto level_dims = MDR::compute_level_dims(dims, (uint32_t)L);
    auto level_elements = MDR::compute_level_elements(level_dims, (uint32_t)L);
    std::vector<uint32_t> dims_dummy(3, 0);
    std::vector<std::vector<uint8_t*>> comps(L + 1);
    std::vector<std::vector<uint32_t>> sizes(L + 1);
    std::vector<std::vector<double>> errs(L + 1);
    std::vector<float> bounds(L + 1);
    int64_t bytes = (int64_t)(N * sizeof(float));
    for (int i = 0; i <= L; i++) {
        const std::vector<uint32_t>& prev = i == 0 ? dims_dummy : level_dims[i - 1];
        std::vector<float> buf(level_elements[i]);
        interleaver.interleave(data.data(), dims, level_dims[i], prev, buf.data());
        const float mx = MDR::compute_max_abs_value(buf.data(), level_elements[i]);
        bounds[i] = mx * 4;
        int exp = 0;
        frexp(mx, &exp);
        comps[i] = encoder.encode(buf.data(), (int32_t)level_elements[i], exp, (uint8_t)B, sizes[i], errs[i]);
        for (uint32_t s : sizes[i]) bytes += s;
    }
    MDR::NegaBinaryGreedyBasedSizeInterpreter<MDR::L2ErrorEstimator_HB<float>> interp(
        MDR::L2ErrorEstimator_HB<float>(3, L));
    std::vector<uint8_t> nbp(L + 1, 0);
    std::vector<float> rec(N, 0.f), cur(N);
    std::vector<uint32_t> strides = {dims[1] * dims[2], dims[2], 1};
    for (int t = 0; t < ntol; t++) {
        std::vector<uint8_t> prev_nbp(nbp);
        interp.interpret_retrieve_size(sizes, errs, tols[t], nbp);
        std::fill(cur.begin(), cur.end(), 0.f);
        for (int i = 0; i <= L; i++) {
            if (nbp[i] > prev_nbp[i]) {
                int exp = 0;
                frexp(bounds[i] / 4, &exp);
                std::vector<const uint8_t*> planes(comps[i].begin() + prev_nbp[i], comps[i].end());
                float* dec = encoder.progressive_decode(planes, (int32_t)level_elements[i], exp, prev_nbp[i],
                                                        (uint8_t)(nbp[i] - prev_nbp[i]), i);
                const std::vector<uint32_t>& prev = i == 0 ? dims_dummy : level_dims[i - 1];
                interleaver.reposition(dec, dims, level_dims[i], prev, cur.data(), strides);
                free(dec);
            }
            for (int p = 0; p < nbp[i]; p++) bytes += sizes[i][p];
        }
        decomposer.recompose(cur.data(), dims, (uint32_t)L, strides);
        for (size_t k = 0; k < N; k++) rec[k] += cur[k];
        bytes += (int64_t)(N * sizeof(float));
    }
    if (out) std::memcpy(out, rec.data(), N * sizeof(float));
    for (auto& c : comps)
        for (auto* p : c) free(p);
    return bytes;
}

// AdaptiveLevelCompressor (zstd, level 3) on B streams concatenated in blob:
// returns the stopping index; out_sizes = the sizes it leaves (compressed or
// raw); zstd_sizes = ZSTD::compress's size of every stream on its own
int ref_adaptive_compress(const uint8_t* blob, const uint32_t* sizes, int B, int latter, uint32_t* out_sizes,
                          uint32_t* zstd_sizes) {
    std::vector<uint8_t*> st(B);
    std::vector<uint32_t> sz(sizes, sizes + B);
    size_t o = 0;
    for (int p = 0; p < B; p++) {
        st[p] = (uint8_t*)malloc(sizes[p] ? sizes[p] : 1);
        std::memcpy(st[p], blob + o, sizes[p]);
        uint8_t* c = nullptr;
        zstd_sizes[p] = MDR::ZSTD::compress(blob + o, sizes[p], &c);
        free(c);
        o += sizes[p];
    }
    MDR::AdaptiveLevelCompressor comp(latter);
    const int stop = comp.compress_level(st, sz);
    for (int p = 0; p < B; p++) { out_sizes[p] = sz[p]; free(st[p]); }
    return stop;
}

// GE quantities of interest (qoi_utils.hpp:135-165) and the pointwise error
// estimates the GE retrieval drivers form with the propagation rules of
// qoi_utils.hpp:18-98: V_TOT as in halving_Vtot.cpp:38-45, T = P / (D R) as in
// UniformTighteningT with c_1 = 1 / R
void ref_qoi_values_f64(const double* vx, const double* vy, const double* vz, const double* p, const double* d,
                        uint64_t n, double* vtot, double* temp, double* c, double* mach, double* pt, double* mu) {
    QoI::compute_QoIs(vx, vy, vz, p, d, (size_t)n, vtot, temp, c, mach, pt, mu);
}
void ref_qoi_vtot_bound_f64(const double* vx, const double* vy, const double* vz, uint64_t n, double ebx, double eby,
                            double ebz, double* out) {
    for (uint64_t i = 0; i < n; i++) {
        double e2 = QoI::compute_bound_x_square(vx[i], ebx) + QoI::compute_bound_x_square(vy[i], eby) +
                    QoI::compute_bound_x_square(vz[i], ebz);
        double v2 = vx[i] * vx[i] + vy[i] * vy[i] + vz[i] * vz[i];
        out[i] = QoI::compute_bound_square_root_x(v2, e2);
    }
}
void ref_qoi_t_bound_f64(const double* p, const double* d, uint64_t n, double ebp, double ebd, double* out) {
    Quiet q;   // the division rule prints a warning where it cannot bound the error
    const double c1 = 1.0 / 287.1;
    for (uint64_t i = 0; i < n; i++) out[i] = c1 * QoI::compute_bound_division(p[i], d[i], ebp, ebd);
}
}
