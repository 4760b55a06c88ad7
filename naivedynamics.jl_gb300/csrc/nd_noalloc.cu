// nd_noalloc.cu -- the pair-list pipeline for callers that cannot allocate
// device memory.
//
// nd_leaf_pairs_noalloc_dev runs the same Morton / radix-sort / tree / rope-walk
// kernels as nd_leaf_pairs_dev, but every scratch buffer is a slice of one
// file-scope device array instead of memory obtained with cudaMalloc.  Callers
// that cannot allocate are, for example, code running inside a host runtime
// that owns the whole device memory budget through its own pool (a GPU array
// package or a framework's caching allocator), or a time-critical loop in which
// cudaMalloc / cudaFree would stall the device.  They pass positions and output
// buffers; the library never grows anything.
//
// Limits and sharing rules (also stated in include/naivegpu.h):
//   * at most kNoAllocMaxAtoms atoms, atomsperleaf >= 2 in both modes (an
//     unordered request with a leaf width other than 4 is served by the
//     ordered emission); larger requests are rejected with ND_ERR_ARG before
//     any work is enqueued;
//   * the array (kNoAllocBytes, ~5.3 MB) is reserved on every GPU that loads
//     the library and stays there until the process exits;
//   * all calls share the one array, so calls whose work overlaps on the GPU
//     (different streams, or different host threads) race and corrupt each
//     other -- serialise them;
//   * the first call on a device looks the array's device address up
//     (cudaGetSymbolAddress, with that device current) and keeps it for the
//     life of the process; make that first call before any stream capture.
//     The kept address does not survive cudaDeviceReset (the module, and with
//     it the array, is loaded again afterwards): no call after a reset.
#include <mutex>

#include "nd_internal.cuh"

namespace {

constexpr int32_t kNoAllocMaxAtoms = 65536;
constexpr int32_t kMaxLeaves = kNoAllocMaxAtoms / 2;  // atomsperleaf >= 2

constexpr size_t up256(size_t b) { return (b + 255) & ~size_t(255); }

// Slice sizes: exactly what the pipeline asks ensure() for at the limits.
constexpr size_t kCodesB = up256(4ull * kNoAllocMaxAtoms);               // codes, perm, alt x2
constexpr size_t kPos4B = up256(16ull * kNoAllocMaxAtoms);               // sorted float4
constexpr size_t kIdxB = up256(4ull * kNoAllocMaxAtoms);                 // sorted index
constexpr size_t kKeysB = up256(32ull * (2 * kMaxLeaves));               // GridKeys
constexpr size_t kStoreB = up256(4ull * kMaxLeaves);                     // CAS slots
constexpr size_t kHistB = up256(4ull * (256 * ((kNoAllocMaxAtoms + 2047) / 2048) + 256));
constexpr size_t kCountsB = up256(8ull * (kMaxLeaves + 1));
constexpr size_t kOffsetsB = up256(8ull * (kMaxLeaves + 2));
constexpr size_t kPartialB = up256(8ull * (4 * ((kMaxLeaves + 4095) / 4096) + 64));
constexpr size_t kMiscB = 256;
constexpr size_t kErrB = 256;
constexpr size_t kNoAllocBytes = 4 * kCodesB + kPos4B + kIdxB + kKeysB + kStoreB + kHistB +
                                 kCountsB + kOffsetsB + kPartialB + kMiscB + kErrB;

// The scratch array.  In host code this name is only a stand-in for the
// symbol; its device address comes from cudaGetSymbolAddress.
static __device__ __align__(256) unsigned char g_nd_noalloc_scratch[kNoAllocBytes];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
void* g_scratch_addr[kMaxDevices] = {};

// Once per device, with that device current: the array's device address.
nd_status scratch_for_current_device(void** out) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
        cudaGetLastError();
        return ND_ERR_NODEVICE;
    }
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_addr[dev]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_nd_noalloc_scratch);
        if (e != cudaSuccess || !p) {
            cudaGetLastError();
            return ND_ERR_CUDA;
        }
        g_scratch_addr[dev] = p;
    }
    *out = g_scratch_addr[dev];
    return ND_OK;
}

void carve(nd::DevBuf& b, unsigned char*& cur, size_t bytes) {
    b.p = cur;
    b.bytes = bytes;
    cur += bytes;
}

}  // namespace

extern "C" nd_status nd_leaf_pairs_noalloc_dev(const float* xyz, const nd_bvh_spec* spec,
                                               int32_t order, int32_t mode, int32_t* pi,
                                               int32_t* pj, float* pd, int64_t capacity,
                                               int64_t* count, void* stream) {
    if (!xyz || !spec || !count || capacity < 0) return ND_ERR_ARG;
    if (spec->atom_count > kNoAllocMaxAtoms || spec->atomsperleaf < 2) return ND_ERR_ARG;
    void* base = nullptr;
    nd_status st = scratch_for_current_device(&base);
    if (st) return st;
    nd::Ctx c;
    c.no_alloc = true;
    cudaGetDevice(&c.device);
    c.stream = (cudaStream_t)stream;
    int32_t h_err[nd::kErrWords] = {0, 0, 0, 0};
    c.h_err = h_err;
    unsigned char* cur = (unsigned char*)base;
    carve(c.codes, cur, kCodesB);
    carve(c.perm, cur, kCodesB);
    carve(c.codes_alt, cur, kCodesB);
    carve(c.perm_alt, cur, kCodesB);
    carve(c.pos4, cur, kPos4B);
    carve(c.idx, cur, kIdxB);
    carve(c.keys, cur, kKeysB);
    carve(c.store, cur, kStoreB);
    carve(c.hist, cur, kHistB);
    carve(c.counts, cur, kCountsB);
    carve(c.offsets, cur, kOffsetsB);
    carve(c.partial, cur, kPartialB);
    carve(c.misc, cur, kMiscB);
    c.d_err = (int32_t*)cur;
    // The previous call may have left an error word or a pair cursor behind;
    // everything else the pipeline reads it writes first (codes, keys and CAS
    // slots are reset by the pipeline itself).
    cudaError_t e = cudaMemsetAsync(c.d_err, 0, kErrB, c.stream);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return ND_ERR_CUDA;
    }
    return nd::pairs_common(&c, spec, order, mode, 0, xyz, false, pi, pj, pd, capacity, count);
}
