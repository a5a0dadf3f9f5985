// Registry of the col tile FFT kernels listed in kernel_list.inc.
#include "kernels.cuh"

#define ESTL_X_TC_SINGLE(M, C) \
  static_assert(SingleKernel<M, 4, 4, C, true>::SMEM_ELEMS * 8 <= kMaxSmemBytes, "tensor-core tile too large");
#define ESTL_X_TC_COL(M, C) \
  static_assert(ColKernel<M, 4, 4, C, true>::SMEM_ELEMS * 8 <= kMaxSmemBytes, "tensor-core tile too large");
#define ESTL_X_TC_ROW(M, C) \
  static_assert(RowKernel<M, 4, 4, C, true>::SMEM_ELEMS * 8 <= kMaxSmemBytes, "tensor-core tile too large");
#define ESTL_X_BULK_COL(M, E, R, C) \
  static_assert(BulkColKernel<M, E, R, C>::SMEM_ELEMS * 8 <= kMaxSmemBytes, "tensor-copy tile too large");
namespace estl {
#include "kernel_list.inc"
}

namespace estl {

static const KernelDesc kTable[] = {
#define ESTL_X_COL(M, E, R, C) ESTL_COL(M, E, R, C),
#define ESTL_X_BULK_COL(M, E, R, C) ESTL_BULK_COL(M, E, R, C),
#define ESTL_X_TC_COL(M, C) ESTL_TC_COL(M, C),
#define ESTL_X_COLUMN(M, E, C) ESTL_COLUMN(M, E, C),
#include "kernel_list.inc"
};

int registry_col(const KernelDesc** out) {
  *out = kTable;
  return (int)(sizeof(kTable) / sizeof(kTable[0]));
}

}  // namespace estl
