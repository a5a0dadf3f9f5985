// Registry of the single tile FFT kernels listed in kernel_list.inc.
#include "kernels.cuh"

namespace estl {

static const KernelDesc kTable[] = {
#define ESTL_X_SINGLE(M, E, R, C) ESTL_SINGLE(M, E, R, C),
#include "kernel_list.inc"
};

int registry_single(const KernelDesc** out) {
  *out = kTable;
  return (int)(sizeof(kTable) / sizeof(kTable[0]));
}

}  // namespace estl
