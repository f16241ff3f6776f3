// Minimal stand-in for the reference's CUDATL::CUDAArray (not shipped in the
// reference tree): ras_qm_mask.h only names it in the signature of its
// table-initialisation function, which the host driver never calls.
#pragma once
#include <cstddef>
namespace CUDATL {
template <class T>
class CUDAArray {
  public:
    void resizeWithoutCopy(size_t n) { n_ = n; }
    T *gptr() { return nullptr; }
    size_t size() const { return n_; }

  private:
    size_t n_ = 0;
};
}  // namespace CUDATL
