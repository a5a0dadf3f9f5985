// kernels.cuh — __global__ wrappers and the kernel registry entries for the
// tile FFT kernels of fft_core.cuh.
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>

#include "fft_core.cuh"
#include "bulk_core.cuh"
#include "resident_core.cuh"
#include "cluster_core.cuh"

namespace estl {

// equal to the planner's StepKind values
enum KernelKind { KIND_SINGLE = 0, KIND_COL = 1, KIND_ROW = 2, KIND_COLUMN = 5 };

struct KernelDesc {
  int kind;
  int logm, loge, logr, logc;
  int nthreads;
  int smem_bytes;
  const void* fn;
  int pipe;  // 0: plain tile; 2: bulk-load ring (bulk_core.cuh);
             // 3 / 4: resident whole transforms with a whole / half exchange buffer (resident_core.cuh)
  int tc;    // radix-16 passes on the tensor cores (tc_core.cuh)
  int tmap;  // launched with a 2D tensor map of its input as a second parameter (tma_tile_kernel)
  int cluster = 0;  // cluster tiles (cluster_core.cuh): log2 CTAs per cluster
  int csplit = 0;   // cluster tiles: log2 of the column DFT length N2
};

template <class K>
__global__ void __launch_bounds__(K::NT, K::MIN_BLOCKS) tile_kernel(TileArgs a) {
  extern __shared__ float2 estl_smem[];
  pdl_wait();
  if constexpr (!is_persistent<K>::value) pdl_trigger();
  K::run(a, (long long)blockIdx.x, (int)threadIdx.x, reinterpret_cast<cf32*>(estl_smem));
}

// Kernels whose tile loads are tensor copies: the map lives in parameter space
// for the whole launch, and the tile code finds it through TileArgs::tmap.
template <class K>
__global__ void __launch_bounds__(K::NT, K::MIN_BLOCKS) tma_tile_kernel(TileArgs a, const __grid_constant__ CUtensorMap map) {
  extern __shared__ float2 estl_smem[];
  pdl_wait();
  if constexpr (!is_persistent<K>::value) pdl_trigger();
  a.tmap = &map;
  K::run(a, (long long)blockIdx.x, (int)threadIdx.x, reinterpret_cast<cf32*>(estl_smem));
}

template <class K>
KernelDesc make_desc(int kind, int logm, int loge, int logr, int logc, int pipe = 0, int tc = 0) {
  return KernelDesc{kind, logm, loge, logr, logc, K::NT, (int)(K::SMEM_ELEMS * sizeof(cf32)),
                    reinterpret_cast<const void*>(&tile_kernel<K>), pipe, tc, 0, cluster_of<K>::log_cluster,
                    cluster_of<K>::log_split};
}

template <class K>
KernelDesc make_tma_desc(int kind, int logm, int loge, int logr, int logc) {
  return KernelDesc{kind, logm, loge, logr, logc, K::NT, (int)(K::SMEM_ELEMS * sizeof(cf32)),
                    reinterpret_cast<const void*>(&tma_tile_kernel<K>), 2, 0, 1};
}

constexpr long long kMaxSmemBytes = 227 * 1024;

#define ESTL_SINGLE(M, E, R, C) make_desc<SingleKernel<M, E, R, C>>(KIND_SINGLE, M, E, R, C)
#define ESTL_COL(M, E, R, C) make_desc<ColKernel<M, E, R, C>>(KIND_COL, M, E, R, C)
#define ESTL_ROW(M, E, R, C) make_desc<RowKernel<M, E, R, C>>(KIND_ROW, M, E, R, C)
#define ESTL_BULK_ROW(M, E, R, C) make_desc<BulkRowKernel<M, E, R, C>>(KIND_ROW, M, E, R, C, 2)
#define ESTL_BULK_COL(M, E, R, C) make_tma_desc<BulkColKernel<M, E, R, C>>(KIND_COL, M, E, R, C)
#define ESTL_RES(M, E, R, H) make_desc<ResKernel<M, E, R, H>>(KIND_SINGLE, M, E, R, 0, 2 + H)
#define ESTL_CLUSTER_TILE(N, LR, N2, E) make_desc<ClusterKernel<N, LR, N2, E>>(KIND_SINGLE, N, E, 4, 0)
#define ESTL_COLUMN(M, E, C) make_desc<ColKernel<M, E, 4, C, false, false>>(KIND_COLUMN, M, E, 4, C)
#define ESTL_TC_SINGLE(M, C) make_desc<SingleKernel<M, 4, 4, C, true>>(KIND_SINGLE, M, 4, 4, C, 0, 1)
#define ESTL_TC_COL(M, C) make_desc<ColKernel<M, 4, 4, C, true>>(KIND_COL, M, 4, 4, C, 0, 1)
#define ESTL_TC_ROW(M, C) make_desc<RowKernel<M, 4, 4, C, true>>(KIND_ROW, M, 4, 4, C, 0, 1)

// Per translation unit tables (kernels_*.cu).
int registry_single(const KernelDesc** out);
int registry_col(const KernelDesc** out);
int registry_row(const KernelDesc** out);

}  // namespace estl
