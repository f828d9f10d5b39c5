// Allocation-free SES field entry point.
//
// Some callers cannot allocate GPU memory while they run: plugins that live inside a host
// application whose memory manager owns every device allocation (game engines, molecular
// viewers), real-time loops that must not hit cudaMalloc's implicit synchronisation, and
// callers with a fixed device-memory budget.  qses_field_codes_noalloc serves them: the
// caller passes device input and output buffers and the function allocates nothing.  Its
// working memory is the file-scope array below, reserved once when the library is loaded
// on a device and held by every GPU that loads the library until the process exits.
//
// The array is shared by all calls: each call clears what must start at zero, and calls
// that overlap on the GPU (different streams or host threads at the same time) race on it.
#include <cuda.h>  // driver API types only: the entry points are looked up at run time
#include <cuda_runtime.h>

#include <cstring>
#include <mutex>
#include <string>

#include "kernels.h"
#include "prims.h"
#include "qses_context.h"

namespace {

constexpr unsigned kNaMaxAtoms = 4096;   // atoms per call
constexpr int kNaMaxG = 128;             // SES voxels per axis
constexpr int kNaMaxGnb = 40;            // neighbour cells per axis
constexpr size_t kNaMaxWords = (size_t)kNaMaxG * kNaMaxG * ((kNaMaxG + 31) / 32);

constexpr size_t al(size_t b) { return (b + 255) & ~(size_t)255; }
constexpr size_t kOffErr = 64;
constexpr size_t kOffKeys = 256;
constexpr size_t kOffAtoms = kOffKeys + 4 * al(4ull * kNaMaxAtoms);
constexpr size_t kOffCells = kOffAtoms + al(16ull * kNaMaxAtoms);
constexpr size_t kOffMasks = kOffCells + al(8ull * kNaMaxGnb * kNaMaxGnb * kNaMaxGnb);
constexpr size_t kOffCodes = kOffMasks + 3 * al(4 * kNaMaxWords);
constexpr size_t kOffTmp = kOffCodes + al((size_t)kNaMaxG * kNaMaxG * kNaMaxG);
constexpr size_t kTmpBytes = 16384;
constexpr size_t kNaBytes = kOffTmp + kTmpBytes;  // about 3.5 MB

// The scratch.  In host code this name is only a stand-in for the device symbol: the host
// passes the address obtained from cudaGetSymbolAddress, never the name itself.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNaBytes];

std::mutex g_na_mu;
void *g_na_addr[64] = {nullptr};          // device address of the scratch, per device ordinal
unsigned long long g_na_ctx[64] = {0};    // the CUDA context that address belongs to
unsigned g_na_bounds[8];                  // host copy of the bounds read-back

// Unique id of the calling thread's current CUDA context (0 if none can be had).  A
// device's primary context can be destroyed and created again (cudaDeviceReset, or a
// library that releases it); the scratch then lives at a new address, so the cached one is
// valid only for the context it was looked up in.  Context ids are never reused, unlike
// context handles.
unsigned long long current_context_id() {
    typedef CUresult (*GetCurrent)(CUcontext *);
    typedef CUresult (*GetId)(CUcontext, unsigned long long *);
    static GetCurrent get_current = nullptr;
    static GetId get_id = nullptr;
    static bool looked_up = false;
    if (!looked_up) {
        cudaDriverEntryPointQueryResult q1, q2;
        void *f1 = nullptr, *f2 = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000, cudaEnableDefault, &q1) == cudaSuccess &&
            cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2) == cudaSuccess &&
            q1 == cudaDriverEntryPointSuccess && q2 == cudaDriverEntryPointSuccess) {
            get_current = (GetCurrent)f1;
            get_id = (GetId)f2;
        }
        cudaGetLastError();
        looked_up = true;
    }
    CUcontext c = nullptr;
    unsigned long long id = 0;
    if (!get_current || !get_id || get_current(&c) != CUDA_SUCCESS || !c || get_id(c, &id) != CUDA_SUCCESS) return 0;
    return id;
}

}  // namespace

extern "C" QSES_API int qses_field_codes_noalloc(const float *d_xyz, const float *d_radii, unsigned n, float voxel,
                                                 uint8_t *d_codes, size_t codes_bytes, void *cuda_stream) {
    using namespace qses;
    if (!d_xyz || !d_radii || !d_codes || n < 2) return QSES_ERR_INVALID_ARG;
    if (n > kNaMaxAtoms) return QSES_ERR_UNSUPPORTED;  // more atoms than the scratch holds
    std::lock_guard<std::mutex> lock(g_na_mu);
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return QSES_ERR_NO_DEVICE;
    const unsigned long long ctx_id = current_context_id();  // 0 before the runtime made one
    if (!g_na_addr[dev] || ctx_id == 0 || ctx_id != g_na_ctx[dev]) {
        // Set-up, once per device (and again only if the device's context was replaced),
        // with the device current: the only host-side use of the symbol.  It is not a
        // stream operation, but it may load the library's module on first use, so the first
        // call on a device should come before any stream capture.
        void *ptr = nullptr;
        if (cudaGetSymbolAddress(&ptr, g_noalloc_scratch) != cudaSuccess || !ptr) {
            cudaGetLastError();
            return QSES_ERR_CUDA;
        }
        g_na_addr[dev] = ptr;
        g_na_ctx[dev] = current_context_id();  // the context the look-up ran in
    }
    char *base = (char *)g_na_addr[dev];
    cudaStream_t s = (cudaStream_t)cuda_stream;
    // Every return after the first enqueue waits for this call's queued work first, so the
    // next call (which may come from another thread once the lock is released) never finds
    // the scratch still in use by this one.
    auto fail = [s](int rc) {
        cudaStreamSynchronize(s);
        cudaGetLastError();
        return rc;
    };

    // Bounds and grid sizing, exactly as the allocating path computes them.
    unsigned *d_mm = (unsigned *)base;
    int *d_err = (int *)(base + kOffErr);
    if (cudaMemsetAsync(d_mm, 0xff, 3 * sizeof(unsigned), s) != cudaSuccess ||
        cudaMemsetAsync(d_mm + 3, 0, 5 * sizeof(unsigned), s) != cudaSuccess ||
        cudaMemsetAsync(d_err, 0, sizeof(int), s) != cudaSuccess)
        return fail(QSES_ERR_CUDA);
    launch_atom_minmax(d_xyz, d_radii, n, d_mm, s);
    if (cudaMemcpyAsync(g_na_bounds, d_mm, sizeof(g_na_bounds), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
        return fail(QSES_ERR_CUDA);
    // From here until the next enqueue the stream holds none of this call's work.
    auto dec = [](unsigned e) {
        unsigned b = (e & 0x80000000u) ? (e & 0x7fffffffu) : ~e;
        float f;
        memcpy(&f, &b, 4);
        return f;
    };
    const float mn[3] = {dec(g_na_bounds[0]), dec(g_na_bounds[1]), dec(g_na_bounds[2])};
    const float mx[3] = {dec(g_na_bounds[3]), dec(g_na_bounds[4]), dec(g_na_bounds[5])};
    QGrid g;
    int rc = grid_from_bounds(mn, mx, dec(g_na_bounds[6]), n, voxel, g, nullptr, nullptr);
    if (rc != QSES_OK) return rc;
    if (g.G > kNaMaxG || g.gnb > kNaMaxGnb) return QSES_ERR_UNSUPPORTED;  // grid larger than the scratch
    const size_t G = (size_t)g.G;
    if (codes_bytes < G * G * G) return QSES_ERR_INVALID_ARG;

    // Carve the scratch; everything that must start at zero is cleared below.
    unsigned *key = (unsigned *)(base + kOffKeys), *key2 = key + al(4ull * kNaMaxAtoms) / 4;
    unsigned *idx = key2 + al(4ull * kNaMaxAtoms) / 4, *idx2 = idx + al(4ull * kNaMaxAtoms) / 4;
    float4 *atoms = (float4 *)(base + kOffAtoms);
    uint2 *cells = (uint2 *)(base + kOffCells);
    unsigned *inMask = (unsigned *)(base + kOffMasks), *outMask = inMask + al(4 * kNaMaxWords) / 4;
    unsigned *signMask = outMask + al(4 * kNaMaxWords) / 4;
    unsigned char *codes = (unsigned char *)(base + kOffCodes);
    void *tmp = base + kOffTmp;
    const size_t ncell = (size_t)g.gnb * g.gnb * g.gnb;
    const int atom_bits = bits_for(ncell - 1);
    if (radix_sort_tmp_bytes(n, atom_bits) > kTmpBytes) return QSES_ERR_INTERNAL;

    launch_atom_hash(g, d_xyz, n, key, s);
    int alt = 0;
    if (radix_sort<unsigned>(key, key2, idx, idx2, n, atom_bits, true, tmp, d_err, s, nullptr, &alt) != cudaSuccess)
        return fail(QSES_ERR_CUDA);
    const unsigned *skey = alt ? key2 : key, *sidx = alt ? idx2 : idx;
    if (cudaMemsetAsync(cells, 0, 8 * ncell, s) != cudaSuccess) return fail(QSES_ERR_CUDA);
    launch_atom_gather(d_xyz, d_radii, skey, sidx, n, atoms, cells, s);
    launch_sas(g, atoms, cells, inMask, outMask, s);
    launch_edt(g, inMask, outMask, codes, signMask, s);
    // Padded rows (32-voxel words) in the scratch -> tight G*G*G rows for the caller.
    if (cudaMemcpy2DAsync(d_codes, G, codes, (size_t)g.Gp, G, G * G, cudaMemcpyDeviceToDevice, s) != cudaSuccess)
        return fail(QSES_ERR_CUDA);
    int herr = 0;
    if (cudaMemcpyAsync(&g_na_bounds[7], d_err, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
        return fail(QSES_ERR_CUDA);
    memcpy(&herr, &g_na_bounds[7], sizeof(int));
    if (herr) return herr;
    return cudaGetLastError() == cudaSuccess ? QSES_OK : QSES_ERR_CUDA;
}
