// Kernel lookup by (object type, metric).  Each object type's instantiations
// live in their own translation unit so they compile in parallel.
#pragma once
#include <cuda_runtime.h>
#include "device_index.h"

namespace ngtg {

struct ExactConfig;

typedef void (*ExactKernelFn)(DevGraph, const uint4*, uint32_t, const QueryParams*, const uint32_t*, ObjDist*,
                              uint32_t*, QueryStats*, uint32_t*, unsigned long long*, ExactConfig);
typedef void (*LinearKernelFn)(DevGraph, const uint4*, uint32_t, uint32_t, const uint8_t*, float*, uint32_t);

struct FastConfig;
typedef void (*FastKernelFn)(DevGraph, const uint4*, const uint4*, uint32_t, const QueryParams*, const uint32_t*,
                             ObjDist*, uint32_t*, QueryStats*, uint32_t*, uint32_t*, unsigned long long*, FastConfig);

typedef void (*QGKernelFn)(DevGraph, DevQG, const uint4*, uint32_t, const QGParams*, const uint32_t*, ObjDist*,
                           uint32_t*, QueryStats*, uint32_t*, unsigned long long*, ExactConfig);
// Quantized-graph kernel for m subspaces (nullptr above 512) and its shared memory.
QGKernelFn qg_kernel(uint32_t m);
size_t qg_kernel_smem_bytes(uint32_t row_chunks, uint32_t dim, uint32_t m, const ExactConfig& c);

struct QGWideConfig;
typedef void (*QGWideKernelFn)(DevGraph, DevQG, const uint4*, uint32_t, const QGParams*, const uint32_t*, ObjDist*,
                               uint32_t*, QueryStats*, uint32_t*, uint32_t*, QGWideConfig);
// Relaxed-order quantized-graph kernel for m subspaces loading `blocks` (2 or 4) code
// blocks per warp at a time (nullptr above 512 subspaces, or 256 with 4) and its
// shared memory.
QGWideKernelFn qg_wide_kernel_for(uint32_t m, uint32_t blocks);
size_t qg_wide_kernel_smem_bytes(uint32_t row_chunks, uint32_t dim, uint32_t m, const QGWideConfig& c);

struct QBGConfig;
typedef void (*QBGKernelFn)(DevGraph, DevQG, const uint32_t*, const uint4*, uint32_t, const QBGParams*,
                            const uint32_t*, ObjDist*, uint32_t*, QueryStats*, uint32_t*, unsigned long long*, float*,
                            QBGConfig);
QBGKernelFn qbg_kernel(uint32_t m);
size_t qbg_kernel_smem_bytes(uint32_t row_chunks, uint32_t dim, uint32_t m, const QBGConfig& c);
// The two-step search's blob phase and the refinement (qbg_search.cuh).
typedef void (*QBGScanKernelFn)(DevQG, const uint32_t*, const uint4*, uint32_t, uint32_t, const QBGParams*,
                                const ObjDist*, const uint32_t*, uint32_t, ObjDist*, uint32_t*, QueryStats*, float*,
                                uint32_t, uint32_t);
QBGScanKernelFn qbg_scan_kernel_for(uint32_t m);
size_t qbg_scan_kernel_smem_bytes(uint32_t row_chunks, uint32_t dim, uint32_t m, uint32_t rcap);
typedef void (*QBGRefineKernelFn)(const ObjDist*, const uint32_t*, uint32_t, const float*, uint32_t, const uint4*,
                                  uint32_t, uint32_t, uint32_t, const uint32_t*, uint32_t, uint32_t, ObjDist*,
                                  uint32_t, uint32_t*);
QBGRefineKernelFn qbg_refine_kernel_for(bool uint8_rows);
// The same re-rank over a graph index's float refinement objects with its distance
// (L1, L2, angle, cosine; nullptr for the others).
QBGRefineKernelFn graph_refine_kernel_for(Metric m);

struct WideConfig;
typedef void (*WideKernelFn)(DevGraph, const uint4*, const uint4*, uint32_t, const QueryParams*, const uint32_t*,
                             ObjDist*, uint32_t*, QueryStats*, uint32_t*, uint32_t*, unsigned long long*, WideConfig);
// CTA-per-query batched kernel with `threads` per CTA: 256 for float L2 (bf16,
// 8-bit or fp32 search rows), uint8 L2 and int8-code L2; 128 also for float L2 on
// bf16 or 8-bit rows and for int8-code L2; nullptr otherwise.
WideKernelFn wide_kernel(ObjType ot, Metric m, SearchRows rows, uint32_t threads = 256);
// The CTA-per-query kernel on the objects themselves for the distances other than L2
// (float: L1, cosine, angle, normalized, Poincare, Lorentz; uint8: L1, Hamming,
// Jaccard; float16: L2, L1), 256 threads; nullptr for the rest.
WideKernelFn wide_kernel_native(ObjType ot, Metric m);
// float rows (dpad per row, `dim` valid) -> 8-bit codes rint((x - offset) / scale), 0 past dim
void launch_float_rows_to_sq8(const float* in, uint8_t* out, size_t nrows, uint32_t dpad, uint32_t dim, float offset,
                              float scale, cudaStream_t s);
size_t wide_kernel_smem_bytes(uint32_t row_chunks, const WideConfig& c);

// Batched kernel for (object type, metric); bf16_rows selects the bf16 search
// rows for float objects.  nullptr when unsupported.
// rows_in_flight (rows per lane group the distance loop keeps in flight) and
// ctas_per_sm (the register budget) select an instantiation: (4, 5) for every
// type; (6, 4), (8, 4), (6, 5), (4, 6), (2, 8) for the float/L2 bf16 search.
// 0 = default.  nullptr when the combination is not built.
FastKernelFn fast_kernel(ObjType ot, Metric m, bool bf16_rows, uint32_t rows_in_flight = 4,
                         uint32_t ctas_per_sm = 0);
void launch_float_rows_to_bf16(const void* in, void* out, size_t nfloats, cudaStream_t s);

// Return nullptr when the (type, metric) pair is not supported.
ExactKernelFn exact_kernel_float(Metric m);
ExactKernelFn exact_kernel_half(Metric m);
ExactKernelFn exact_kernel_u8(Metric m);
ExactKernelFn exact_kernel_qs8(Metric m);
LinearKernelFn linear_kernel_float(Metric m);
LinearKernelFn linear_kernel_half(Metric m);
LinearKernelFn linear_kernel_u8(Metric m);
LinearKernelFn linear_kernel_qs8(Metric m);

// Metric used by the kernels: inner product runs as L2 over the augmented rows.
inline Metric kernel_metric(Metric m) { return m == Metric::InnerProduct ? Metric::L2 : m; }

}  // namespace ngtg
