// Registry of the row tile FFT kernels listed in kernel_list.inc.
#include "kernels.cuh"

namespace estl {

static const KernelDesc kTable[] = {
#define ESTL_X_ROW(M, E, R, C) ESTL_ROW(M, E, R, C),
#include "kernel_list.inc"
};

int registry_row(const KernelDesc** out) {
  *out = kTable;
  return (int)(sizeof(kTable) / sizeof(kTable[0]));
}

}  // namespace estl
