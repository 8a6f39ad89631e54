// Compile-time drop-in check: the reference's own ComposedRefactor and
// ComposedReconstructor templates instantiated with the GPU plugin adapters
// (only built where the reference headers are available; never run).
#include <cstdint>
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
    return out ? 0 : 1;
}
