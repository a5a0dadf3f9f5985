// Registry of the col tile FFT kernels listed in kernel_list.inc.
#include "kernels.cuh"

namespace estl {

static const KernelDesc kTable[] = {
#define ESTL_X_COL(M, E, R, C) ESTL_COL(M, E, R, C),
#include "kernel_list.inc"
};

int registry_col(const KernelDesc** out) {
  *out = kTable;
  return (int)(sizeof(kTable) / sizeof(kTable[0]));
}

}  // namespace estl
