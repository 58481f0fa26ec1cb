/* Test-infrastructure stand-in for CUSP's array1d (CUSP is not available):
 * a std::vector with the memory-space tag ignored, so that the reference's
 * domain.h and body.h compile on the host unchanged. */
#pragma once
#include <vector>
namespace cusp {
struct host_memory {};
struct device_memory {};
template <class T, class Mem>
struct array1d : std::vector<T> {
    using std::vector<T>::vector;
};
}  // namespace cusp
