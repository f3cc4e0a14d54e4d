// noalloc.cu -- opx_reduce_noalloc: the BulkQuantities reductions of opx_reduce
// for callers that cannot allocate device memory.
//
// Who needs it: code that embeds this library in a host whose device memory is
// owned by someone else -- a framework with its own caching allocator that
// must see every byte (a cudaMalloc behind its back fragments its pool and can
// fail under its memory cap), a JVM or service process whose GPU budget is
// fixed up front, or a caller in the middle of work that must not stall on the
// implicit device synchronisation of cudaMalloc/cudaFree.  Such a caller
// already holds the fields in its own device buffers and only wants the
// numbers.
//
// How: the per-block partial sums, which opx_reduce keeps in memory allocated
// with its handle, live here in one file-scope __device__ array of fixed size
// (OPX_NOALLOC_BLOCKS blocks x 8 quantities x 2 doubles = 77,824 bytes), held by
// every GPU that loads the library until the process exits.  Host code cannot
// pass the array's name to a kernel (on the host it is only a stand-in, not a
// device address), so the device address is obtained once per device with
// cudaGetSymbolAddress, with that device current, on the first call of the
// entry point on that device; that first call should therefore come before any
// stream capture.  Every call reuses the same array: calls that overlap on the
// GPU (on different streams, or from different host threads) race on it.  Each
// block overwrites its own partials before the final kernel reads them, so no
// part of the array has to start at zero.  The cached address belongs to the
// device's context: after cudaDeviceReset on a device it is stale, so a process
// that resets a device must not call this entry point on that device again.
// Unlike opx_reduce, non-finite field values are not turned into an error
// status; they reach the record as NaN or Inf, and the caller checks it.
#include <mutex>

#include "internal.h"
#include "ksum.cuh"
#include "observables.cuh"

namespace opx {

constexpr int OPX_NOALLOC_BLOCKS = 608;  // 4 blocks per SM on 152 SMs
constexpr long OPX_NOALLOC_MAX_SITES = 1L << 29;

static __device__ __align__(256) double g_noalloc_partials[OPX_NOALLOC_BLOCKS * NQ * 2];

template <int NC, typename R>
__global__ void __launch_bounds__(256) k_noalloc_partial(const R *__restrict__ U, const R *__restrict__ Unext,
                                                         const R *__restrict__ E, const R *__restrict__ rho,
                                                         const uint8_t *__restrict__ eval, Lat L,
                                                         double *__restrict__ part) {
    KSum acc[NQ];
    bulk_accumulate<NC, R>(U, Unext, E, rho, eval, L, acc, (long)blockIdx.x * blockDim.x + threadIdx.x,
                           (long)gridDim.x * blockDim.x);
    int q;
    KSum v = block_reduce<NQ>(acc, q);
    if (q >= 0) {
        part[((long)blockIdx.x * NQ + q) * 2] = v.s;
        part[((long)blockIdx.x * NQ + q) * 2 + 1] = v.c;
    }
}

// Sums the partials in block order and writes an opx_observables record.
__global__ void k_noalloc_final(const double *__restrict__ part, int nblocks, double V,
                                opx_observables *__restrict__ out) {
    __shared__ double tot[NQ];
    const int q = threadIdx.x;
    if (q < NQ) {
        KSum v{0.0, 0.0};
        for (int b = 0; b < nblocks; b++) ksum_merge(v, KSum{part[((long)b * NQ + q) * 2], part[((long)b * NQ + q) * 2 + 1]});
        tot[q] = v.s + v.c;
    }
    __syncthreads();
    if (threadIdx.x != 0) return;
    double es[3], bs[3];
    for (int i = 0; i < 3; i++) {
        es[i] = tot[i] / V;
        bs[i] = tot[3 + i] / V;
        out->e2[i] = es[i];
        out->b2[i] = bs[i];
    }
    out->px = -es[0] + es[1] + es[2] - bs[0] + bs[1] + bs[2];
    out->py = +es[0] - es[1] + es[2] + bs[0] - bs[1] + bs[2];
    out->pz = +es[0] + es[1] - es[2] + bs[0] + bs[1] - bs[2];
    out->gauss = tot[6] / V;
    out->rho2 = sqrt(tot[7]) / V;
    out->e2_total = es[0] + es[1] + es[2];
    out->b2_total = bs[0] + bs[1] + bs[2];
}

static std::mutex g_noalloc_mutex;
static double *g_noalloc_addr[64];  // device address of g_noalloc_partials, per device ordinal

static int noalloc_scratch(double **out) {
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess || dev < 0 || dev >= 64) return OPX_ERR_CUDA;
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (!g_noalloc_addr[dev]) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_partials);
        if (e != cudaSuccess || !p) return OPX_ERR_CUDA;
        g_noalloc_addr[dev] = (double *)p;
    }
    *out = g_noalloc_addr[dev];
    return OPX_OK;
}

template <int NC, typename R>
static void noalloc_launch(const Lat &L, const void *U, const void *Unext, const void *E, const void *rho,
                           const uint8_t *eval, double *part, int nblocks, opx_observables *out,
                           cudaStream_t st) {
    k_noalloc_partial<NC, R><<<nblocks, 256, 0, st>>>((const R *)U, (const R *)Unext, (const R *)E,
                                                      (const R *)rho, eval, L, part);
    k_noalloc_final<<<1, 32, 0, st>>>(part, nblocks, (double)L.V, out);
}

}  // namespace opx

using namespace opx;

extern "C" int opx_reduce_noalloc(int ncolors, int precision, const int *dims, const double *a, double g,
                                  const void *U, const void *Unext, const void *E, const void *rho,
                                  const uint8_t *eval, opx_observables *out_device, void *stream) {
    if ((ncolors != 2 && ncolors != 3) || (precision != OPX_F64 && precision != OPX_F32) || !dims || !a ||
        !U || !Unext || !E || !out_device || !(g > 0))
        return OPX_ERR_INVALID;
    // SU(2) links are read as 16-byte vectors: a misaligned buffer is refused here
    // rather than faulting on the device
    if (((uintptr_t)U | (uintptr_t)Unext) & 15) return OPX_ERR_INVALID;
    long V = 1;
    for (int i = 0; i < 3; i++) {
        if (dims[i] < 1 || !(a[i] > 0)) return OPX_ERR_INVALID;
        V *= dims[i];
        if (V > OPX_NOALLOC_MAX_SITES) return OPX_ERR_INVALID;  // beyond the stated maximum
    }
    double *part = nullptr;
    int rc = noalloc_scratch(&part);
    if (rc) return rc;
    const Lat L = make_lat(dims, a, 1.0, g);
    const int nblocks = (int)std::min<long>((V + 255) / 256, OPX_NOALLOC_BLOCKS);
    cudaStream_t st = (cudaStream_t)stream;
    // an error left pending by earlier work of the caller is neither reported nor cleared here
    const cudaError_t pending = cudaPeekAtLastError();
    if (ncolors == 2) {
        if (precision == OPX_F64) noalloc_launch<2, double>(L, U, Unext, E, rho, eval, part, nblocks, out_device, st);
        else noalloc_launch<2, float>(L, U, Unext, E, rho, eval, part, nblocks, out_device, st);
    } else {
        if (precision == OPX_F64) noalloc_launch<3, double>(L, U, Unext, E, rho, eval, part, nblocks, out_device, st);
        else noalloc_launch<3, float>(L, U, Unext, E, rho, eval, part, nblocks, out_device, st);
    }
    const cudaError_t e = cudaPeekAtLastError();
    if (e != cudaSuccess && e != pending) {
        (void)cudaGetLastError();  // this call's launch error: consumed and reported
        return OPX_ERR_CUDA;
    }
    return OPX_OK;
}
