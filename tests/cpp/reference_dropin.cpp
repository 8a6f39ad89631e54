// Runtime drop-in check (built and run by tests/test_gpu_cpp_plugins.py on a
// GPU host where the reference's headers are available): the reference's own
// ComposedRefactor and ComposedReconstructor templates
// (ComposedRefactor.hpp:21-46, ComposedReconstructor.hpp:106-122) drive the
// GPU plugin adapters of include/prodm_gb300_mdr.hpp end to end.
//  1. The level files and metadata that ComposedRefactor writes with the GPU
//     adapters are byte-identical to the ones it writes with the reference's
//     own CPU components (whose MGARD decomposer is the oracle's restatement),
//     and the level files equal the device-resident GpuComposedRefactor's.
//  2. ComposedReconstructor with the GPU adapters, reading those files,
//     retrieves the same bytes and reconstructs the same level as with the
//     reference's CPU components, its progressive reconstructions equal
//     theirs to float rounding, and every full-resolution one meets its L-inf
//     tolerance.
// Configurations: fp32 negabinary and grouped (MaxErrorCollector,
// SignExclude interpreter, MaxErrorEstimatorHB) and fp64 PerBit with 60
// planes (the GE applications' encoder).
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <iostream>
#include <memory>
#include <queue>
#include <string>
#include <vector>

#include "MDR/Refactor/Refactor.hpp"
#include "MDR/Reconstructor/Reconstructor.hpp"
#include "prodm_gb300_mdr.hpp"

using namespace prodm_gb300;

static std::vector<uint8_t> read_all(const std::string& f) {
    FILE* fp = std::fopen(f.c_str(), "rb");
    if (!fp) return {};
    std::fseek(fp, 0, SEEK_END);
    long n = std::ftell(fp);
    std::rewind(fp);
    std::vector<uint8_t> b(n);
    if (std::fread(b.data(), 1, n, fp) != (size_t)n) b.clear();
    std::fclose(fp);
    return b;
}

template <class T>
static std::vector<T> make_field(size_t n0) {
    std::vector<T> f(n0 * n0 * n0);
    for (size_t i = 0; i < n0; i++)
        for (size_t j = 0; j < n0; j++)
            for (size_t k = 0; k < n0; k++)
                f[(i * n0 + j) * n0 + k] =
                    (T)(std::sin(0.3 * i + 0.1) * std::cos(0.2 * j) + std::sin(0.45 * k + 0.7 * i) + 0.01 * std::cos(1.7 * k * j));
    return f;
}

static std::vector<std::string> names(const std::string& d, const std::string& tag, int L) {
    std::vector<std::string> v;
    for (int l = 0; l <= L; l++) v.push_back(d + "/" + tag + "_level_" + std::to_string(l) + ".bin");
    return v;
}

// GpuEnc / CpuEnc: the adapter and the reference encoder of one configuration;
// Comp: the level compressor; negabinary: the metadata flag ComposedRefactor
// writes (test_mdr_refactor.cpp sets it for the negabinary encoder)
template <class T, class GpuEnc, class CpuEnc, class GpuComp, class CpuComp>
static int run(const std::string& dir, const char* tag, int enc_id, int B, bool negabinary, GpuEnc genc, GpuEnc gdec,
               const std::shared_ptr<StreamSizeTable>& table) {
    const std::vector<uint32_t> dims = {65, 65, 65};
    const int L = 3;
    const size_t N = 65 * 65 * 65;
    std::vector<T> field = make_field<T>(65);
    const std::string tg = std::string(tag);
    auto fg = names(dir, tg + "_gpu", L), fc = names(dir, tg + "_cpu", L), fd = names(dir, tg + "_dev", L);
    const std::string mg = dir + "/" + tg + "_gpu_meta.bin", mc = dir + "/" + tg + "_cpu_meta.bin",
                      md = dir + "/" + tg + "_dev_meta.bin";
    {
        auto r = MDR::ComposedRefactor<T, GpuMGARDHierarchicalDecomposer<T>, GpuDirectInterleaver<T>, GpuEnc, GpuComp,
                                       GpuMaxErrorCollector<T>, MDR::ConcatLevelFileWriter>(
            GpuMGARDHierarchicalDecomposer<T>(), GpuDirectInterleaver<T>(), genc, GpuComp(), GpuMaxErrorCollector<T>(),
            MDR::ConcatLevelFileWriter(mg, fg));
        r.negabinary = negabinary;
        r.refactor(field.data(), dims, L, B);
    }
    {
        auto r = MDR::ComposedRefactor<T, MDR::MGARDHierarchicalDecomposer<T>, MDR::DirectInterleaver<T>, CpuEnc, CpuComp,
                                       MDR::MaxErrorCollector<T>, MDR::ConcatLevelFileWriter>(
            MDR::MGARDHierarchicalDecomposer<T>(), MDR::DirectInterleaver<T>(), CpuEnc(), CpuComp(),
            MDR::MaxErrorCollector<T>(), MDR::ConcatLevelFileWriter(mc, fc));
        r.negabinary = negabinary;
        r.refactor(field.data(), dims, L, B);
    }
    {   // the device path writes the same level files (its metadata adds fields)
        GpuComposedRefactor<T> r(enc_id, PRODM_BASIS_HIERARCHICAL, PRODM_COLLECT_MAX, md, fd);
        r.refactor(field.data(), dims, L, B);
        for (int l = 0; l <= L; l++)
            if (read_all(fg[l]) != read_all(fd[l])) {
                std::printf("%s: level %d differs between the adapters and the device path\n", tag, l);
                return 1;
            }
    }
    for (int l = 0; l <= L; l++) {
        const auto a = read_all(fg[l]);
        if (a.empty() || a != read_all(fc[l])) {
            std::printf("%s: level %d file differs between GPU adapters and the reference's CPU components\n", tag, l);
            return 1;
        }
    }
    if (read_all(mg) != read_all(mc)) {
        std::printf("%s: metadata differs between GPU adapters and the reference's CPU components\n", tag);
        return 1;
    }

    using GInterp = GpuGreedySizeInterpreter<T, PRODM_INTERP_SIGN_EXCLUDE, PRODM_EST_MAX_HB>;
    auto gr = MDR::ComposedReconstructor<T, GpuMGARDHierarchicalDecomposer<T>, GpuDirectInterleaver<T>, GpuEnc, GpuComp,
                                         GInterp, MDR::MaxErrorEstimatorHB<T>, MDR::ConcatLevelFileRetriever>(
        GpuMGARDHierarchicalDecomposer<T>(), GpuDirectInterleaver<T>(), gdec, GpuComp(),
        GInterp(MDR::MaxErrorEstimatorHB<T>(), table), MDR::ConcatLevelFileRetriever(mg, fg));
    using CInterp = MDR::SignExcludeGreedyBasedSizeInterpreter<MDR::MaxErrorEstimatorHB<T>>;
    auto cr = MDR::ComposedReconstructor<T, MDR::MGARDHierarchicalDecomposer<T>, MDR::DirectInterleaver<T>, CpuEnc,
                                         CpuComp, CInterp, MDR::MaxErrorEstimatorHB<T>, MDR::ConcatLevelFileRetriever>(
        MDR::MGARDHierarchicalDecomposer<T>(), MDR::DirectInterleaver<T>(), CpuEnc(), CpuComp(),
        CInterp(MDR::MaxErrorEstimatorHB<T>()), MDR::ConcatLevelFileRetriever(mc, fc));
    gr.load_metadata();
    cr.load_metadata();
    T vmin = field[0], vmax = field[0], mag = 0;
    for (T v : field) {
        vmin = v < vmin ? v : vmin;
        vmax = v > vmax ? v : vmax;
        mag = std::fabs(v) > mag ? std::fabs(v) : mag;
    }
    const double rels[] = {1e-1, 1e-2, 1e-3, 1e-4, 1e-5};
    for (double rel : rels) {
        const double tol = rel * (vmax - vmin);
        std::vector<T> g(N), c(N);
        T* go = gr.progressive_reconstruct(tol, -1);
        if (!go) { std::printf("%s: GPU reconstruction failed\n", tag); return 1; }
        std::memcpy(g.data(), go, N * sizeof(T));
        T* co = cr.progressive_reconstruct(tol, -1);
        std::memcpy(c.data(), co, N * sizeof(T));
        if (gr.get_retrieved_size() != cr.get_retrieved_size()) {
            std::printf("%s: retrieved %zu bytes against the reference's %zu at %g\n", tag, gr.get_retrieved_size(),
                        cr.get_retrieved_size(), tol);
            return 1;
        }
        if (gr.get_reconstruct_level() != cr.get_reconstruct_level()) {
            std::printf("%s: reconstructs level %d against the reference's %d\n", tag, gr.get_reconstruct_level(),
                        cr.get_reconstruct_level());
            return 1;
        }
        double err = 0, diff = 0;
        for (size_t i = 0; i < N; i++) {
            err = std::fmax(err, std::fabs((double)g[i] - field[i]));
            diff = std::fmax(diff, std::fabs((double)g[i] - c[i]));
        }
        const double ftol = (sizeof(T) == 4 ? 1e-5 : 1e-13) * mag;
        if (diff > ftol) { std::printf("%s: differs from the reference's reconstruction by %g\n", tag, diff); return 1; }
        // no planes of the finest levels: the reference reconstructs a coarser
        // level into the array's corner (ComposedReconstructor.hpp:75-90), and
        // the bound applies to full-resolution results only
        const bool full = gr.get_reconstruct_level() == L;
        if (full && err > tol) { std::printf("%s: tolerance %g missed (%g)\n", tag, tol, err); return 1; }
        std::printf("%s tol %.3g: level %d, max error %.3g, retrieved %zu bytes, |gpu - reference| %.3g\n", tag, tol,
                    gr.get_reconstruct_level(), full ? err : 0.0, gr.get_retrieved_size(), diff);
    }
    std::printf("%s ok\n", tag);
    return 0;
}

int main(int argc, char** argv) {
    const std::string dir = argc > 1 ? argv[1] : ".";
    int rc = 0;
    rc |= run<float, GpuNegaBinaryBPEncoder<float, uint32_t>, MDR::NegaBinaryBPEncoder<float, uint32_t>,
              MDR::NullLevelCompressor, MDR::NullLevelCompressor>(
        dir, "negabinary", PRODM_ENC_NEGABINARY, 32, true, GpuNegaBinaryBPEncoder<float, uint32_t>(),
        GpuNegaBinaryBPEncoder<float, uint32_t>(), nullptr);
    rc |= run<float, GpuGroupedBPEncoder<float, uint32_t>, MDR::GroupedBPEncoder<float, uint32_t>,
              MDR::NullLevelCompressor, MDR::NullLevelCompressor>(
        dir, "grouped", PRODM_ENC_GROUPED, 32, false, GpuGroupedBPEncoder<float, uint32_t>(),
        GpuGroupedBPEncoder<float, uint32_t>(), nullptr);
    auto table = std::make_shared<StreamSizeTable>();
    rc |= run<double, GpuPerBitBPEncoder<double, uint32_t>, MDR::PerBitBPEncoder<double, uint32_t>,
              MDR::NullLevelCompressor, MDR::NullLevelCompressor>(
        dir, "perbit", PRODM_ENC_PERBIT, 60, false, GpuPerBitBPEncoder<double, uint32_t>(),
        GpuPerBitBPEncoder<double, uint32_t>(table), table);
    if (rc == 0) std::printf("REFERENCE DROP-IN OK\n");
    return rc;
}
