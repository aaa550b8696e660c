// fdf_noalloc.cu -- fdf_SortByCellNoAlloc: the sort by cell of fdf_SortByCell for
// callers that cannot allocate device memory.
//
// Who needs it: host codes whose device memory is owned by someone else -- a PETSc
// or MPI application that hands this library only the buffers it already has, code
// running where an allocation would block or fail (inside a memory-capped pool, or a
// real-time loop that must not enter the allocator).  They pass the inputs and the
// outputs; the only scratch the sort needs (the per-cell slot cursors and the block
// sums of the scan) lives in the file-scope device array below, which every GPU that
// loads this library holds until the process exits.
//
// Limits and rules:
//  * at most FDF_NOALLOC_MAX_CELLS cells (larger requests return FDF_ERR_ARG_OUTOFRANGE
//    and launch nothing);
//  * at most FDF_MAX_PARTICLES particle slots, as fdf_SortByCell;
//  * the first call on a device looks up the array's device address there
//    (cudaGetSymbolAddress with that device current) and caches it; make that first
//    call outside any stream capture.  The cached address belongs to the device's
//    primary context: a caller that resets the device (cudaDeviceReset) must not call
//    this function afterwards in the same process;
//  * all calls share the one array, and each call clears the part that must start at
//    zero, so results never depend on an earlier call -- but two calls whose work
//    overlaps on the GPU (different streams, or different host threads) race on it:
//    serialise them;
//  * no cudaMalloc, cudaFree or allocating library routine is called.
#include "fdf_internal.cuh"
#include "../../include/fdf_gb300.h"

#include <mutex>

namespace {

constexpr long long NOALLOC_SUMS_WORDS = (FDF_NOALLOC_MAX_CELLS + 1 + 8191) / 8192 + 1;
constexpr long long NOALLOC_CURSOR_WORDS = (FDF_NOALLOC_MAX_CELLS + 63) / 64 * 64;   // keeps sums 256-B aligned
constexpr long long NOALLOC_WORDS = NOALLOC_CURSOR_WORDS + NOALLOC_SUMS_WORDS;

constexpr int MAX_DEVICES = 64;
std::mutex g_setup_mutex;
unsigned int *g_scratch_addr[MAX_DEVICES] = {};

}  // namespace

// The scratch: per-cell cursors, then the scan's block sums.
static __device__ __align__(256) unsigned int g_noalloc_scratch[NOALLOC_WORDS];

namespace {

// Device address of g_noalloc_scratch on the current device (looked up once per device).
int noalloc_scratch(unsigned int **out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return FDF_ERR_GPU;
  if (dev < 0 || dev >= MAX_DEVICES) return FDF_ERR_SUP;
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (!g_scratch_addr[dev]) {
    unsigned int *ptr = nullptr;
    cudaError_t e = cudaGetSymbolAddress((void **)&ptr, g_noalloc_scratch);
    if (e != cudaSuccess || !ptr) return FDF_ERR_GPU;
    g_scratch_addr[dev] = ptr;
  }
  *out = g_scratch_addr[dev];
  return FDF_SUCCESS;
}

}  // namespace

extern "C" int fdf_SortByCellNoAlloc(const int32_t *cell_ids, int64_t n, int64_t ncells, uint32_t *perm,
                                     uint32_t *cell_start, void *stream) {
  if (n > 0 && (!cell_ids || !perm)) return FDF_ERR_ARG_NULL;
  if (!cell_start) return FDF_ERR_ARG_NULL;
  if (n < 0 || n > FDF_MAX_PARTICLES || ncells < 1 || ncells > FDF_NOALLOC_MAX_CELLS) return FDF_ERR_ARG_OUTOFRANGE;
  unsigned int *scratch = nullptr;
  int r = noalloc_scratch(&scratch);
  if (r) return r;
  unsigned int *cursor = scratch;
  unsigned int *sums = scratch + NOALLOC_CURSOR_WORDS;
  cell_sort_on_scratch(cell_ids, n, ncells, perm, cell_start, cursor, sums, (cudaStream_t)stream);
  return cudaGetLastError() == cudaSuccess ? FDF_SUCCESS : FDF_ERR_GPU;
}
