// Runtime check of the C++ plugin adapters (built and run by
// tests/test_gpu_cpp_plugins.py on a GPU host):
//  1. the adapters driven through the steps of ComposedRefactor::refactor
//     (ComposedRefactor.hpp:78-141: decompose, per level interleave -> max ->
//     frexp -> encode) produce level files byte-identical to the
//     device-resident GpuComposedRefactor;
//  2. GpuComposedReconstructor reading those files meets every L-inf
//     tolerance, and the adapter path (interpreter -> progressive_decode ->
//     reposition -> recompose, ComposedReconstructor.hpp:187-258) matches it
//     to float rounding.
#include <cmath>
#include <cstdint>
#include <memory>
#include <type_traits>
#include <cstdio>
#include <string>
#include <vector>

#include "prodm_gb300_mdr.hpp"

struct MDR_EST_TAG {};   // stands for the estimator object the reference interpreters take

// decoders: the per-bit adapter takes the shared size table, the others not
template <class E>
static E make_decoder(std::shared_ptr<prodm_gb300::StreamSizeTable> t) {
    if constexpr (std::is_same<E, prodm_gb300::GpuPerBitBPEncoder<double, uint32_t>>::value) return E(t);
    else return E();
}

using namespace prodm_gb300;

static std::vector<uint8_t> read_all(const std::string& f) {
    FILE* fp = std::fopen(f.c_str(), "rb");
    std::fseek(fp, 0, SEEK_END);
    long n = std::ftell(fp);
    std::rewind(fp);
    std::vector<uint8_t> b(n);
    if (std::fread(b.data(), 1, n, fp) != (size_t)n) std::abort();
    std::fclose(fp);
    return b;
}

// Enc: encoder id; EncT: its adapter class. The per-bit run decodes twice:
// stream sizes from the table the interpreter fills, and found by the host walk
template <class T, int Enc, class EncT>
static int run(const char* dir, const char* tag, int B) {
    const std::vector<uint32_t> dims = {65, 65, 65};
    const int L = 3;
    const size_t N = 65 * 65 * 65;
    std::vector<T> field(N);
    for (size_t i = 0; i < 65; i++)
        for (size_t j = 0; j < 65; j++)
            for (size_t k = 0; k < 65; k++)
                field[(i * 65 + j) * 65 + k] = (T)(std::sin(0.3 * i + 0.1) * std::cos(0.2 * j) + std::sin(0.45 * k + 0.7 * i));
    std::string d(dir);
    std::vector<std::string> files;
    for (int l = 0; l <= L; l++) files.push_back(d + "/" + tag + "_level_" + std::to_string(l) + ".bin");
    const std::string meta = d + "/" + tag + "_metadata.bin";

    // 1. adapters through the ComposedRefactor steps
    GpuMGARDHierarchicalDecomposer<T> dec;
    GpuDirectInterleaver<T> il;
    EncT enc;
    std::vector<T> data(field);
    dec.decompose(data.data(), dims, L);
    std::vector<std::vector<uint32_t>> ld(L + 1, std::vector<uint32_t>(3));
    for (int dd = 0; dd < 3; dd++) {
        uint32_t n = dims[dd];
        for (int j = 0; j <= L; j++) { ld[L - j][dd] = n; n = (n >> 1) + 1; }
    }
    std::vector<std::vector<uint8_t>> adapter_files(L + 1);
    std::vector<std::vector<uint32_t>> level_sizes(L + 1);
    std::vector<T> bounds(L + 1);
    size_t prev = 0;
    for (int l = 0; l <= L; l++) {
        const size_t box = (size_t)ld[l][0] * ld[l][1] * ld[l][2];
        const size_t n = box - prev;
        prev = box;
        std::vector<uint32_t> coarse = l ? ld[l - 1] : std::vector<uint32_t>(3, 0);
        std::vector<T> buf(n);
        il.interleave(data.data(), dims, ld[l], coarse, buf.data());
        T mx = 0;
        for (T v : buf) mx = std::fabs(v) > mx ? std::fabs(v) : mx;
        bounds[l] = Enc == PRODM_ENC_NEGABINARY ? mx * 4 : mx;
        int e = 0;
        std::frexp(mx, &e);
        std::vector<uint32_t> sizes;
        auto streams = enc.encode(buf.data(), (int32_t)n, e, B, sizes);
        level_sizes[l] = sizes;
        for (int p = 0; p < B; p++) {
            adapter_files[l].insert(adapter_files[l].end(), streams[p], streams[p] + sizes[p]);
            std::free(streams[p]);
        }
    }
    GpuComposedRefactor<T> ref(Enc, PRODM_BASIS_HIERARCHICAL, PRODM_COLLECT_MAX, meta, files);
    ref.refactor(field.data(), dims, L, B);
    for (int l = 0; l <= L; l++) {
        if (read_all(files[l]) != adapter_files[l]) {
            std::printf("%s: level %d file differs between adapters and device path\n", tag, l);
            return 1;
        }
    }

    // 2. reconstruction: device path vs adapter path
    const int interp = PRODM_INTERP_SIGN_EXCLUDE;
    GpuComposedReconstructor<T> rec(Enc, PRODM_BASIS_HIERARCHICAL, interp, PRODM_EST_MAX_HB, meta, files);
    rec.load_metadata();
    auto table = std::make_shared<StreamSizeTable>();
    GpuGreedySizeInterpreter<T, PRODM_INTERP_SIGN_EXCLUDE, PRODM_EST_MAX_HB> gi(MDR_EST_TAG(), table);
    EncT pdec = make_decoder<EncT>(table);
    EncT wdec = make_decoder<EncT>(nullptr);   // per-bit: sizes by the host walk
    pdec.set_total_bitplanes(B);
    wdec.set_total_bitplanes(B);
    GpuMaxErrorCollector<T> mc;
    std::vector<std::vector<double>> lerr(L + 1);
    for (int l = 0; l <= L; l++) lerr[l] = mc.collect_level_error(nullptr, 0, B, bounds[l]);
    std::vector<uint8_t> index(L + 1, 0);
    std::vector<T> acc(N, 0);          // accumulated coefficients (in-place layout)
    T vmin = field[0], vmax = field[0];
    for (T v : field) { vmin = v < vmin ? v : vmin; vmax = v > vmax ? v : vmax; }
    for (double rel : {1e-1, 1e-2, 1e-3, 1e-4, 1e-5}) {
        const double tol = rel * (vmax - vmin);
        T* out = rec.progressive_reconstruct(tol);
        double err = 0;
        for (size_t i = 0; i < N; i++) err = std::fmax(err, std::fabs((double)out[i] - field[i]));
        if (err > tol) { std::printf("%s: tolerance %g missed (%g)\n", tag, tol, err); return 1; }
        std::vector<uint8_t> prev_index(index);
        gi.interpret_retrieve_size(level_sizes, lerr, tol, index);
        for (int l = 0; l <= L; l++) {
            const int num = index[l] - prev_index[l];
            if (num <= 0) continue;
            std::vector<const uint8_t*> st;
            size_t off = 0;
            for (int p = 0; p < prev_index[l]; p++) off += level_sizes[l][p];
            for (int p = prev_index[l]; p < index[l]; p++) { st.push_back(adapter_files[l].data() + off); off += level_sizes[l][p]; }
            int e = 0;
            std::frexp(Enc == PRODM_ENC_NEGABINARY ? bounds[l] / 4 : bounds[l], &e);
            const size_t box = (size_t)ld[l][0] * ld[l][1] * ld[l][2];
            const size_t pbox = l ? (size_t)ld[l - 1][0] * ld[l - 1][1] * ld[l - 1][2] : 0;
            T* lv = pdec.progressive_decode(st, (int32_t)(box - pbox), e, prev_index[l], num, l);
            if (Enc == PRODM_ENC_PERBIT) {
                T* lw = wdec.progressive_decode(st, (int32_t)(box - pbox), e, prev_index[l], num, l);
                const bool same = std::memcmp(lv, lw, (box - pbox) * sizeof(T)) == 0;
                std::free(lw);
                if (!same) { std::printf("%s: table and walked stream sizes decode differently\n", tag); return 1; }
            }
            std::vector<uint32_t> coarse = l ? ld[l - 1] : std::vector<uint32_t>(3, 0);
            std::vector<T> cur(N, 0);
            il.reposition(lv, dims, ld[l], coarse, cur.data());
            std::free(lv);
            for (size_t i = 0; i < N; i++) acc[i] += cur[i];
        }
        std::vector<T> full(acc);
        dec.recompose(full.data(), dims, L);
        double diff = 0, mag = 0;
        for (size_t i = 0; i < N; i++) { diff = std::fmax(diff, std::fabs((double)full[i] - out[i])); mag = std::fmax(mag, std::fabs((double)field[i])); }
        if (diff > 1e-5 * mag) { std::printf("%s: adapter path differs from device path by %g\n", tag, diff); return 1; }
    }
    std::printf("%s ok\n", tag);
    return 0;
}

// the lossless stage: GpuComposedRefactor with it on writes the level files
// the adapters produce with GpuAdaptiveLevelCompressor::compress_level, and
// GpuComposedReconstructor reading them meets every tolerance
static int run_lossless(const char* dir) {
    using T = float;
    const std::vector<uint32_t> dims = {65, 65, 65};
    const int L = 3, B = 32;
    const size_t N = 65 * 65 * 65;
    std::vector<T> field(N);
    for (size_t i = 0; i < N; i++) field[i] = (T)(std::sin(0.001 * i) + 0.01 * std::cos(0.37 * i));
    std::string d(dir);
    std::vector<std::string> files;
    for (int l = 0; l <= L; l++) files.push_back(d + "/lossless_level_" + std::to_string(l) + ".bin");
    const std::string meta = d + "/lossless_metadata.bin";
    GpuComposedRefactor<T> ref(PRODM_ENC_GROUPED, PRODM_BASIS_HIERARCHICAL, PRODM_COLLECT_MAX, meta, files);
    ref.set_lossless(26);
    ref.refactor(field.data(), dims, L, B);
    GpuMGARDHierarchicalDecomposer<T> dec;
    GpuDirectInterleaver<T> il;
    GpuGroupedBPEncoder<T, uint32_t> enc;
    GpuAdaptiveLevelCompressor comp;
    std::vector<T> data(field);
    dec.decompose(data.data(), dims, L);
    std::vector<std::vector<uint32_t>> ld(L + 1, std::vector<uint32_t>(3));
    for (int dd = 0; dd < 3; dd++) {
        uint32_t n = dims[dd];
        for (int j = 0; j <= L; j++) { ld[L - j][dd] = n; n = (n >> 1) + 1; }
    }
    size_t prev = 0;
    for (int l = 0; l <= L; l++) {
        const size_t box = (size_t)ld[l][0] * ld[l][1] * ld[l][2];
        const size_t n = box - prev;
        prev = box;
        std::vector<uint32_t> coarse = l ? ld[l - 1] : std::vector<uint32_t>(3, 0);
        std::vector<T> buf(n);
        il.interleave(data.data(), dims, ld[l], coarse, buf.data());
        T mx = 0;
        for (T v : buf) mx = std::fabs(v) > mx ? std::fabs(v) : mx;
        int e = 0;
        std::frexp(mx, &e);
        std::vector<uint32_t> sizes;
        auto streams = enc.encode(buf.data(), (int32_t)n, e, B, sizes);
        std::vector<uint32_t> raw(sizes);
        std::vector<uint8_t*> keep(B);
        for (int p = 0; p < B; p++) {   // copies for the round trip below
            keep[p] = (uint8_t*)std::malloc(sizes[p] ? sizes[p] : 1);
            std::memcpy(keep[p], streams[p], sizes[p]);
        }
        const uint8_t stop = comp.compress_level(streams, sizes);
        std::vector<uint8_t> bytes;
        for (int p = 0; p < B; p++) {
            bytes.insert(bytes.end(), streams[p], streams[p] + sizes[p]);
        }
        if (read_all(files[l]) != bytes) { std::printf("lossless: level %d file differs from the adapters'\n", l); return 1; }
        std::vector<const uint8_t*> cst(streams.begin(), streams.end());
        comp.decompress_level(cst, sizes, 0, (uint8_t)B, stop);
        for (int p = 0; p < B; p++) {
            if (std::memcmp(cst[p], keep[p], raw[p]) != 0) { std::printf("lossless: level %d plane %d round trip\n", l, p); return 1; }
            std::free(keep[p]);
            std::free(streams[p]);
        }
        comp.decompress_release();
    }
    GpuComposedReconstructor<T> rec(PRODM_ENC_GROUPED, PRODM_BASIS_HIERARCHICAL, PRODM_INTERP_SIGN_EXCLUDE,
                                    PRODM_EST_MAX_HB, meta, files);
    rec.load_metadata();
    T vmin = field[0], vmax = field[0];
    for (T v : field) { vmin = v < vmin ? v : vmin; vmax = v > vmax ? v : vmax; }
    for (double rel : {1e-1, 1e-3, 1e-5}) {
        const double tol = rel * (vmax - vmin);
        T* out = rec.progressive_reconstruct(tol);
        double err = 0;
        for (size_t i = 0; i < N; i++) err = std::fmax(err, std::fabs((double)out[i] - field[i]));
        if (err > tol) { std::printf("lossless: tolerance %g missed (%g)\n", tol, err); return 1; }
    }
    std::printf("lossless ok\n");
    return 0;
}

int main(int argc, char** argv) {
    const char* dir = argc > 1 ? argv[1] : ".";
    int rc = run<float, PRODM_ENC_NEGABINARY, GpuNegaBinaryBPEncoder<float, uint32_t>>(dir, "negabinary", 32);
    rc |= run<float, PRODM_ENC_GROUPED, GpuGroupedBPEncoder<float, uint32_t>>(dir, "grouped", 32);
    rc |= run<double, PRODM_ENC_PERBIT, GpuPerBitBPEncoder<double, uint32_t>>(dir, "perbit", 60);
    rc |= run_lossless(dir);
    if (rc == 0) std::printf("PLUGIN PARITY OK\n");
    return rc;
}
