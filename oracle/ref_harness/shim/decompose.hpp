// Stand-in for MGARDx's decompose.hpp (github.com/lxAltria/MGARDx, absent from
// this tree): forwards to the oracle's own restatement of the MGARD transform.
#pragma once
#include <vector>
#include <cstddef>
#include "../../mdr_oracle.hpp"
namespace MGARD {
template <class T>
class Decomposer {
public:
    void decompose(T* data, const std::vector<size_t>& dims, size_t target_level, bool hierarchical,
                   std::vector<size_t> strides = std::vector<size_t>()) {
        std::vector<uint32_t> d(dims.begin(), dims.end()), s(strides.begin(), strides.end());
        mdr_oracle::decompose<T>(data, d, (int)target_level, hierarchical, s);
    }
};
}  // namespace MGARD
