// noalloc.cu - cell-table compaction that allocates no device memory.
//
// pbf_launch_cell_ranges_compact needs a few KB of scratch (a tile counter
// and one look-back status word per tile of sorted keys), which its caller
// allocates and passes in.  Some callers cannot do that while they run: a
// host application's frame loop in which cudaMalloc / cudaFree would
// synchronize the device and stall the frame, or a plugin host that budgets
// all GPU memory itself and hands its plugins none.  For them this file keeps
// the scratch in one fixed device array that exists as soon as the library is
// loaded on a GPU (every GPU that loads the library holds it until the
// process exits), and the entry point below uses it.
//
// Limits and sharing:
//   * at most kNoAllocMaxKeys sorted keys per call (larger calls are refused
//     with PBF_ERR_UNSUPPORTED, nothing is launched);
//   * every call, from every thread and stream, uses the same array; the
//     call clears what must start at zero (tile counter, status words, error
//     word) before its kernel runs, so leftovers of an earlier call do not
//     matter, but two calls whose work overlaps on the GPU race on the array
//     and give wrong tables.  Serialize them (one stream, or events).
#include <cstdint>
#include <mutex>

#include "../../include/pbf/pbf.h"
#include "grid.cuh"

namespace {

// 16,777,216 keys: 256 B header + one 4-byte status word per compaction tile.
constexpr uint32_t kNoAllocMaxKeys = 1u << 24;
constexpr size_t kNoAllocTiles = (size_t(kNoAllocMaxKeys) + pbf::kCompactTile - 1) / pbf::kCompactTile;
constexpr size_t kNoAllocScratchBytes = 256 + ((kNoAllocTiles * 4u + 255u) & ~size_t(255));

static __device__ __align__(256) unsigned char g_compact_scratch[kNoAllocScratchBytes];

// Device address of g_compact_scratch, looked up with the device current (the
// host-side symbol is only a stand-in and must never be handed to a kernel).
// It is cached per device together with the context it was looked up in:
// after cudaDeviceReset the device gets a new context, the module is loaded
// again and the array may move, so a changed context means a new lookup.  The
// context is read through the driver entry point the runtime hands out, so
// the library needs no link against the driver library.
constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
struct ScratchSlot {
    void* ctx = nullptr;
    void* addr = nullptr;
};
ScratchSlot g_scratch[kMaxDevices];

using CtxGetCurrentFn = int (*)(void**);  // CUresult cuCtxGetCurrent(CUcontext*)
CtxGetCurrentFn g_ctx_get_current = nullptr;

int current_context(void** ctx) {
    if (!g_ctx_get_current) {
        void* fn = nullptr;
        cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
        // cuCtxGetCurrent has had one signature since CUDA 4.0
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &fn, 4000, cudaEnableDefault, &q) != cudaSuccess ||
            q != cudaDriverEntryPointSuccess || !fn)
            return PBF_ERR_CUDA;
        g_ctx_get_current = reinterpret_cast<CtxGetCurrentFn>(fn);
    }
    *ctx = nullptr;
    return g_ctx_get_current(ctx) == 0 ? PBF_OK : PBF_ERR_CUDA;  // null: no context current yet
}

int scratch_address(void** out) {
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return PBF_ERR_CUDA;
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    void* ctx = nullptr;
    int st = current_context(&ctx);
    if (st != PBF_OK) return st;
    ScratchSlot& slot = g_scratch[dev];
    if (!ctx || !slot.addr || slot.ctx != ctx) {
        // the lookup also makes the device's primary context current (and
        // loads this library's module in it) if that has not happened yet
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_compact_scratch);
        if (e != cudaSuccess || p == nullptr) return PBF_ERR_CUDA;
        st = current_context(&ctx);
        if (st != PBF_OK || !ctx) return PBF_ERR_CUDA;
        slot.ctx = ctx;
        slot.addr = p;
    }
    *out = slot.addr;
    return PBF_OK;
}

}  // namespace

extern "C" int pbf_launch_cell_ranges_compact_noalloc(uint32_t* uniqueKeys, uint32_t* offsets, uint32_t* compactCount,
                                                      const uint32_t* keysSorted, uint32_t N, cudaStream_t s) {
    if (N > kNoAllocMaxKeys) return PBF_ERR_UNSUPPORTED;
    if (!offsets || !compactCount) return PBF_ERR_INVALID;
    if (N > 0 && (!uniqueKeys || !keysSorted)) return PBF_ERR_INVALID;
    if (pbf::compact_scratch_bytes(N) > kNoAllocScratchBytes) return PBF_ERR_UNSUPPORTED;
    void* scratch = nullptr;
    const int st = scratch_address(&scratch);
    if (st != PBF_OK) return st;
    const cudaError_t e = pbf::launch_compact(scratch, kNoAllocScratchBytes, uniqueKeys, offsets, compactCount, nullptr,
                                              keysSorted, N, s, nullptr);
    if (e == cudaSuccess) return PBF_OK;
    return e == cudaErrorMemoryAllocation ? PBF_ERR_OOM : PBF_ERR_CUDA;
}
