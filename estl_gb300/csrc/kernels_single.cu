// Registry of the single tile FFT kernels listed in kernel_list.inc.
#include "kernels.cuh"

#define ESTL_X_TC_SINGLE(M, C) \
  static_assert(SingleKernel<M, 4, 4, C, true>::SMEM_ELEMS * 8 <= kMaxSmemBytes, "tensor-core tile too large");
#define ESTL_X_RES(M, E, R, H) \
  static_assert(ResKernel<M, E, R, H>::SMEM_ELEMS * 8 <= kMaxSmemBytes, "resident tile too large");
#define ESTL_X_CLUSTER(N, LR, N2, E) \
  static_assert(ClusterKernel<N, LR, N2, E>::SMEM_ELEMS * 8 <= kMaxSmemBytes, "cluster tile too large");
#define ESTL_X_TC_COL(M, C) \
  static_assert(ColKernel<M, 4, 4, C, true>::SMEM_ELEMS * 8 <= kMaxSmemBytes, "tensor-core tile too large");
#define ESTL_X_TC_ROW(M, C) \
  static_assert(RowKernel<M, 4, 4, C, true>::SMEM_ELEMS * 8 <= kMaxSmemBytes, "tensor-core tile too large");
namespace estl {
#include "kernel_list.inc"
}

namespace estl {

static const KernelDesc kTable[] = {
#define ESTL_X_SINGLE(M, E, R, C) ESTL_SINGLE(M, E, R, C),
#define ESTL_X_TC_SINGLE(M, C) ESTL_TC_SINGLE(M, C),
#define ESTL_X_RES(M, E, R, H) ESTL_RES(M, E, R, H),
#define ESTL_X_CLUSTER(N, LR, N2, E) ESTL_CLUSTER_TILE(N, LR, N2, E),
#include "kernel_list.inc"
};

int registry_single(const KernelDesc** out) {
  *out = kTable;
  return (int)(sizeof(kTable) / sizeof(kTable[0]));
}

}  // namespace estl
