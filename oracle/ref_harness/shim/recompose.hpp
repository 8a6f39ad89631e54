// Stand-in for MGARDx's recompose.hpp: forwards to the oracle's restatement.
#pragma once
#include <vector>
#include <cstddef>
#include "../../mdr_oracle.hpp"
namespace MGARD {
template <class T>
class Recomposer {
public:
    void recompose(T* data, const std::vector<size_t>& dims, size_t target_level, bool hierarchical,
                   std::vector<size_t> strides = std::vector<size_t>()) {
        std::vector<uint32_t> d(dims.begin(), dims.end()), s(strides.begin(), strides.end());
        mdr_oracle::recompose<T>(data, d, (int)target_level, hierarchical, s);
    }
};
}  // namespace MGARD
