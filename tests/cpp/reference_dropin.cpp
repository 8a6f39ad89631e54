// Compile-time drop-in check: the reference's own ComposedRefactor and
// ComposedReconstructor templates instantiated with the GPU plugin adapters
// (only built where the reference headers are available; never run).
#include <cstdint>
#include <memory>
#include <iostream>
#include <vector>
#include <string>
#include <cstring>
#include <cmath>
#include <queue>
#include "MDR/Refactor/Refactor.hpp"
#include "MDR/Reconstructor/Reconstructor.hpp"
#include "prodm_gb300_mdr.hpp"

using namespace prodm_gb300;

int main() {
    using T = float;
    std::vector<std::string> files = {"l0.bin", "l1.bin"};
    auto refactor = MDR::ComposedRefactor<T, GpuMGARDHierarchicalDecomposer<T>, GpuDirectInterleaver<T>,
                                          GpuNegaBinaryBPEncoder<T, uint32_t>, MDR::NullLevelCompressor,
                                          GpuSquaredErrorCollector<T>, MDR::ConcatLevelFileWriter>(
        GpuMGARDHierarchicalDecomposer<T>(), GpuDirectInterleaver<T>(), GpuNegaBinaryBPEncoder<T, uint32_t>(),
        MDR::NullLevelCompressor(), GpuSquaredErrorCollector<T>(), MDR::ConcatLevelFileWriter("meta.bin", files));
    std::vector<T> data(33 * 33 * 33, 1.0f);
    refactor.refactor(data.data(), {33, 33, 33}, 1, 32);
    using Interp = GpuGreedySizeInterpreter<T, PRODM_INTERP_SIGN_EXCLUDE, PRODM_EST_MAX_HB>;
    auto rec = MDR::ComposedReconstructor<T, GpuMGARDHierarchicalDecomposer<T>, GpuDirectInterleaver<T>,
                                          GpuGroupedBPEncoder<T, uint32_t>, MDR::NullLevelCompressor, Interp,
                                          MDR::MaxErrorEstimatorHB<T>, MDR::ConcatLevelFileRetriever>(
        GpuMGARDHierarchicalDecomposer<T>(), GpuDirectInterleaver<T>(), GpuGroupedBPEncoder<T, uint32_t>(),
        MDR::NullLevelCompressor(), Interp(MDR::MaxErrorEstimatorHB<T>()), MDR::ConcatLevelFileRetriever("meta.bin", files));
    rec.load_metadata();
    T* out = rec.progressive_reconstruct(1e-3, -1);

    // the GE applications' configuration: per-bit encoder, fp64, max collector;
    // the interpreter hands the metadata stream sizes to the per-bit decoder
    using D = double;
    std::vector<std::string> gfiles = {"g0.bin", "g1.bin"};
    auto grefactor = MDR::ComposedRefactor<D, GpuMGARDHierarchicalDecomposer<D>, GpuDirectInterleaver<D>,
                                           GpuPerBitBPEncoder<D, uint32_t>, MDR::NullLevelCompressor,
                                           GpuMaxErrorCollector<D>, MDR::ConcatLevelFileWriter>(
        GpuMGARDHierarchicalDecomposer<D>(), GpuDirectInterleaver<D>(), GpuPerBitBPEncoder<D, uint32_t>(),
        MDR::NullLevelCompressor(), GpuMaxErrorCollector<D>(), MDR::ConcatLevelFileWriter("gmeta.bin", gfiles));
    std::vector<D> gdata(33 * 33 * 33, 1.0);
    grefactor.refactor(gdata.data(), {33, 33, 33}, 1, 60);
    auto table = std::make_shared<StreamSizeTable>();
    using GInterp = GpuGreedySizeInterpreter<D, PRODM_INTERP_SIGN_EXCLUDE, PRODM_EST_MAX_HB>;
    auto grec = MDR::ComposedReconstructor<D, GpuMGARDHierarchicalDecomposer<D>, GpuDirectInterleaver<D>,
                                           GpuPerBitBPEncoder<D, uint32_t>, MDR::NullLevelCompressor, GInterp,
                                           MDR::MaxErrorEstimatorHB<D>, MDR::ConcatLevelFileRetriever>(
        GpuMGARDHierarchicalDecomposer<D>(), GpuDirectInterleaver<D>(), GpuPerBitBPEncoder<D, uint32_t>(table),
        MDR::NullLevelCompressor(), GInterp(MDR::MaxErrorEstimatorHB<D>(), table),
        MDR::ConcatLevelFileRetriever("gmeta.bin", gfiles));
    grec.load_metadata();
    D* gout = grec.progressive_reconstruct(1e-6, -1);

    // the lossless stage as the composed classes' compressor
    auto lrefactor = MDR::ComposedRefactor<T, GpuMGARDHierarchicalDecomposer<T>, GpuDirectInterleaver<T>,
                                           GpuGroupedBPEncoder<T, uint32_t>, GpuAdaptiveLevelCompressor,
                                           GpuMaxErrorCollector<T>, MDR::ConcatLevelFileWriter>(
        GpuMGARDHierarchicalDecomposer<T>(), GpuDirectInterleaver<T>(), GpuGroupedBPEncoder<T, uint32_t>(),
        GpuAdaptiveLevelCompressor(), GpuMaxErrorCollector<T>(), MDR::ConcatLevelFileWriter("lmeta.bin", files));
    lrefactor.refactor(data.data(), {33, 33, 33}, 1, 32);
    auto lrec = MDR::ComposedReconstructor<T, GpuMGARDHierarchicalDecomposer<T>, GpuDirectInterleaver<T>,
                                           GpuGroupedBPEncoder<T, uint32_t>, GpuAdaptiveLevelCompressor, Interp,
                                           MDR::MaxErrorEstimatorHB<T>, MDR::ConcatLevelFileRetriever>(
        GpuMGARDHierarchicalDecomposer<T>(), GpuDirectInterleaver<T>(), GpuGroupedBPEncoder<T, uint32_t>(),
        GpuAdaptiveLevelCompressor(), Interp(MDR::MaxErrorEstimatorHB<T>()),
        MDR::ConcatLevelFileRetriever("lmeta.bin", files));
    lrec.load_metadata();
    T* lout = lrec.progressive_reconstruct(1e-3, -1);
    return out && gout && lout ? 0 : 1;
}
