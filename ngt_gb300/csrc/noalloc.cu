// Graph search that allocates no device memory.
//
// Some callers cannot allocate GPU memory while they search: plugin hosts
// that own and budget all device memory themselves (a database engine or an
// inference server with its own pool), and latency-critical serving paths that
// must never enter the CUDA allocator, whose calls can block or synchronise the
// device.  ngtgpu_search_exact_noalloc serves them: it
// runs the exact-order graph search kernel with all of its scratch memory -- the
// per-call query parameters and seed lists, and each CTA's visited bitmap and
// candidate overflow tier -- carved from the fixed array below instead of from
// cudaMalloc.  The caller still passes (and owns) the query rows, the result
// buffers and the stream.
//
// The array is a file-scope __device__ variable.  CUDA loads the module that
// holds it lazily, so the 32 MiB are reserved on a GPU when the module is first
// used there; the library does that while it opens an index on that GPU (the
// array's address lookup below), so from then until the process exits the GPU
// holds the array, and the search itself triggers no module load.  Host code
// cannot use the name as a device pointer (it denotes a host-side shadow), so
// the device address is looked up once per device with cudaGetSymbolAddress,
// with that device current.  All calls share the array and it keeps the
// previous call's contents, so each call clears what must start at zero (the
// visited bitmaps); calls whose work overlaps on the GPU (on different
// streams, or from different threads) race on it.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <mutex>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "engine.h"

extern "C" {
#include "../../include/ngtgpu.h"
}

namespace ngtg {

// Maximum scratch of the no-allocation search: 32 MiB per GPU.
constexpr size_t kNoAllocScratchBytes = 32u << 20;
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

namespace {
std::mutex g_scratch_mu;
void* g_scratch_addr[256] = {};
}  // namespace

// Device address of the scratch array on `device` (which must be current).
// The first call on a device performs the lookup, which loads the array's module
// and so reserves the array on that device.
void* noalloc_scratch_address(int device) {
  std::lock_guard<std::mutex> lock(g_scratch_mu);
  if (device < 0 || device >= 256) throw std::runtime_error("device ordinal out of range");
  if (!g_scratch_addr[device]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess)
      throw std::runtime_error(std::string("cudaGetSymbolAddress of the no-allocation scratch failed: ") +
                               cudaGetErrorString(e));
    g_scratch_addr[device] = p;
  }
  return g_scratch_addr[device];
}

size_t noalloc_scratch_bytes() { return kNoAllocScratchBytes; }

void noalloc_prepare_device(int device, const void* exact_fn) {
  noalloc_scratch_address(device);
  cudaFuncAttributes attr;
  cudaError_t e = cudaFuncGetAttributes(&attr, exact_fn);     // loads the kernel's module
  if (e != cudaSuccess)
    throw std::runtime_error(std::string("loading the exact search kernel failed: ") + cudaGetErrorString(e));
}

}  // namespace ngtg

extern "C" bool ngtgpu_search_exact_noalloc(NGTIndex index, const void* d_rows, size_t nq,
                                            const NGTQueryParameters* params, size_t nparams,
                                            NGTObjectDistance* d_results, size_t kmax, uint32_t* d_counts,
                                            NGTGPUQueryStats* d_stats, void* stream, NGTError error) {
  auto fail = [&](const std::string& msg) {
    std::stringstream ss;
    ss << "Capi : " << __FUNCTION__ << "() : Error: " << msg;
    if (error) *static_cast<std::string*>(error) = ss.str();
    else fprintf(stderr, "%s\n", ss.str().c_str());
    return false;
  };
  if (index == nullptr || (nq && (d_rows == nullptr || d_results == nullptr || d_counts == nullptr ||
                                  d_stats == nullptr)) ||
      params == nullptr || !(nparams == 1 || nparams == nq))
    return fail("parametor error: index, buffers or the number of parameter blocks");
  try {
    ngtg::GraphEngine* e = static_cast<ngtg::GraphEngine*>(index);
    std::vector<ngtg::SearchArgs> a(nparams);
    for (size_t i = 0; i < nparams; i++) {
      int es = (int)params[i].edge_size;
      a[i].size = params[i].size;
      a[i].epsilon = params[i].epsilon;
      a[i].radius = params[i].radius < 0.0f ? 3.402823466e+38f : params[i].radius;
      a[i].edge_size = es == INT32_MIN ? -1 : es;
    }
    cudaError_t ce = cudaSetDevice(e->device());
    if (ce != cudaSuccess) return fail(std::string("cudaSetDevice: ") + cudaGetErrorString(ce));
    void* scratch = ngtg::noalloc_scratch_address(e->device());
    cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : e->stream();
    e->search_device_noalloc(scratch, ngtg::noalloc_scratch_bytes(), static_cast<const uint4*>(d_rows), nq,
                             a.data(), a.size(), reinterpret_cast<ngtg::ObjDist*>(d_results), d_counts,
                             reinterpret_cast<ngtg::QueryStats*>(d_stats), kmax, s);
    return true;
  } catch (std::exception& ex) {
    return fail(ex.what());
  }
}
