// batch_kernels.cu -- many independent lattices ("events") of uneven sizes
// stepped together: the batching form of the leapfrog.
//
// The reference runs one Simulation per event; a batch of MV-model ensembles
// or uneven lattices is a loop over independent Simulations.  Here all events
// advance in one persistent launch:
//   * events are assigned to thread-block clusters by longest-processing-time
//     scheduling on their site counts (host side, opx_batch_run);
//   * a cluster owns its events for every step of the launch: its CTAs split
//     each event's sites, and the hardware cluster barrier separates the steps
//     (no grid-wide barrier, no spin-wait: clusters never wait for each other);
//   * the launch is captured once in a CUDA graph and replayed;
//   * the cluster size and block size are picked by timing the candidates on
//     the batch itself (opx_batch_autotune).
// The per-site arithmetic is the single-lattice one (leapfrog.cuh).
#include <cooperative_groups.h>

#include <algorithm>
#include <map>
#include <numeric>
#include <string>
#include <tuple>
#include <vector>

#include "internal.h"
#include "ksum.cuh"
#include "leapfrog.cuh"
#include "observables.cuh"
#include "su3_pair.cuh"

namespace cg = cooperative_groups;

namespace opx {

template <typename R> struct BEvent {
    Lat L;
    R *B[2];  // link buffers: U = B[cur], Unext = B[cur ^ 1]
    R *E;
};

// Step k of a launch starting with U = B[cur] reads B[cur ^ ((k + 1) & 1)] (the
// links after storeFields) and writes B[cur ^ (k & 1)] (Unext).
// I is the type of the site and element offsets (int when every event's fit).
template <int NC, typename R, typename I>
__global__ void __launch_bounds__(256) k_batch_persistent(const BEvent<R> *__restrict__ ev,
                                                          const int *__restrict__ list,
                                                          const int *__restrict__ begin, int nsteps, int cur,
                                                          long step0, int reunit_every) {
    cg::cluster_group cluster = cg::this_cluster();
    const unsigned csize = cluster.num_blocks();
    const unsigned rank = cluster.block_rank();
    const int cid = blockIdx.x / csize;
    const int e0 = begin[cid], e1 = begin[cid + 1];
    const I first = (I)rank * (I)blockDim.x + (I)threadIdx.x;
    const I stride = (I)csize * (I)blockDim.x;
    for (int k = 0; k < nsteps; k++) {
        const bool reunit = reunit_every > 0 && ((step0 + k + 1) % reunit_every) == 0;
        const int rd = cur ^ ((k + 1) & 1), wr = cur ^ (k & 1);
        for (int q = e0; q < e1; q++) {
            const BEvent<R> &e = ev[list[q]];
            const R *U = e.B[rd];
            R *Un = e.B[wr];
            for (I s = first; s < (I)e.L.V; s += stride) {
                // SU(2): the plane-by-plane staple sums, as the flat schedule and
                // the single-lattice kernel (so that every schedule gives the same bits)
                if constexpr (NC == 2) {
                    if (reunit) update_site_su2_planes<R, false, true, I>(U, e.E, nullptr, Un, e.L, s);
                    else update_site_su2_planes<R, false, false, I>(U, e.E, nullptr, Un, e.L, s);
                } else {
                    if (reunit) update_site<NC, R, false, true, I>(U, e.E, nullptr, Un, e.L, s);
                    else update_site<NC, R, false, false, I>(U, e.E, nullptr, Un, e.L, s);
                }
            }
        }
        cluster.sync();
    }
}

// SU(3) FP32: the paired form of the single-lattice kernel (two sites per
// thread in paired FP32 instructions, su3_pair.cuh).  Thread slot t of an
// event covers sites sa = 64 (t / 32) + t % 32 and sb = sa + 32.
template <typename I>
__global__ void __launch_bounds__(128, 3) k_batch_persistent_su3f(const BEvent<float> *__restrict__ ev,
                                                                  const int *__restrict__ list,
                                                                  const int *__restrict__ begin, int nsteps,
                                                                  int cur, long step0, int reunit_every) {
    cg::cluster_group cluster = cg::this_cluster();
    const unsigned csize = cluster.num_blocks();
    const unsigned rank = cluster.block_rank();
    const int cid = blockIdx.x / csize;
    const int e0 = begin[cid], e1 = begin[cid + 1];
    const I first = (I)rank * (I)blockDim.x + (I)threadIdx.x;
    const I stride = (I)csize * (I)blockDim.x;
    for (int k = 0; k < nsteps; k++) {
        const bool reunit = reunit_every > 0 && ((step0 + k + 1) % reunit_every) == 0;
        const int rd = cur ^ ((k + 1) & 1), wr = cur ^ (k & 1);
        for (int q = e0; q < e1; q++) {
            const BEvent<float> &e = ev[list[q]];
            const float *U = e.B[rd];
            float *Un = e.B[wr];
            const I V = (I)e.L.V, slots = ((V + 63) >> 6) << 5;
            for (I t = first; t < slots; t += stride) {
                const I sa = ((t >> 5) << 6) + (t & 31);
                if (sa >= V) continue;
                I sb = sa + 32;
                const bool vb = sb < V;
                if (!vb) sb = sa;
                if (reunit) update_site_pair<I, false, true>(U, e.E, nullptr, Un, e.L, sa, sb, true, vb);
                else update_site_pair<I, false, false>(U, e.E, nullptr, Un, e.L, sa, sb, true, vb);
            }
        }
        cluster.sync();
    }
}

// Flat schedule: one launch per step over the sites of all events, each block
// inside one event (blocks of event order[q] start at bstart[q]; events in
// decreasing size), no cluster.  The hardware block scheduler balances the
// load, and a step costs one launch (replayed from a CUDA graph) instead of a
// cluster barrier.  rd: the buffer holding U (Unext is rd ^ 1).
__device__ __forceinline__ int flat_event(const int *__restrict__ bstart, int nev, int b) {
    int lo = 0, hi = nev - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (__ldg(bstart + mid) <= b) lo = mid; else hi = mid - 1;
    }
    return lo;
}

// blocks of 256 threads per SM the generic flat kernel is compiled for (SU(2)
// FP32: 64 registers, as the single-lattice kernel)
template <int NC, typename R> struct FlatBounds { static constexpr int minb = 1; };
template <> struct FlatBounds<2, float> { static constexpr int minb = 4; };

template <int NC, typename R, typename I, bool REUNIT>
__global__ void __launch_bounds__(256, FlatBounds<NC, R>::minb) k_batch_flat(const BEvent<R> *__restrict__ ev, const int *__restrict__ order,
                                                    const int *__restrict__ bstart, int nev, int rd) {
    const int q = flat_event(bstart, nev, (int)blockIdx.x);
    const BEvent<R> &e = ev[order[q]];
    const I s = (I)((int)blockIdx.x - bstart[q]) * (I)blockDim.x + (I)threadIdx.x;
    if (s >= (I)e.L.V) return;
    if constexpr (NC == 2) update_site_su2_planes<R, false, REUNIT, I>(e.B[rd], e.E, nullptr, e.B[rd ^ 1], e.L, s);
    else update_site<NC, R, false, REUNIT, I>(e.B[rd], e.E, nullptr, e.B[rd ^ 1], e.L, s);
}

// SU(3) FP32, paired: thread slot t of an event covers sa = 64 (t / 32) + t % 32, sb = sa + 32
template <typename I, bool REUNIT>
__global__ void __launch_bounds__(128, 3) k_batch_flat_su3f(const BEvent<float> *__restrict__ ev,
                                                            const int *__restrict__ order,
                                                            const int *__restrict__ bstart, int nev, int rd) {
    const int q = flat_event(bstart, nev, (int)blockIdx.x);
    const BEvent<float> &e = ev[order[q]];
    const I t = (I)((int)blockIdx.x - bstart[q]) * (I)blockDim.x + (I)threadIdx.x;
    const I V = (I)e.L.V, sa = ((t >> 5) << 6) + (t & 31);
    if (sa >= V) return;
    I sb = sa + 32;
    const bool vb = sb < V;
    if (!vb) sb = sa;
    update_site_pair<I, false, REUNIT>(e.B[rd], e.E, nullptr, e.B[rd ^ 1], e.L, sa, sb, true, vb);
}

template <int NC, typename R, typename I, bool REUNIT> static void *flat_kernel() {
    if constexpr (NC == 3 && sizeof(R) == 4) return (void *)k_batch_flat_su3f<I, REUNIT>;
    else return (void *)k_batch_flat<NC, R, I, REUNIT>;
}

// the persistent kernel of a batch's group and precision
template <int NC, typename R, typename I> static void *persistent_kernel() {
    if constexpr (NC == 3 && sizeof(R) == 4) return (void *)k_batch_persistent_su3f<I>;
    else return (void *)k_batch_persistent<NC, R, I>;
}

template <int NC, typename R>
__global__ void k_batch_links(const BEvent<R> *__restrict__ ev, int nev, int cur) {
    const int q = blockIdx.y;
    if (q >= nev) return;
    const BEvent<R> &e = ev[q];
    for (long s = (long)blockIdx.x * blockDim.x + threadIdx.x; s < e.L.V; s += (long)gridDim.x * blockDim.x)
        update_links_site<NC, R>(e.B[cur], e.E, e.B[cur ^ 1], e.L, s);
}

constexpr int BATCH_RED_CHUNKS = 16;

template <int NC, typename R>
__global__ void __launch_bounds__(256) k_batch_bulk(const BEvent<R> *__restrict__ ev, int cur,
                                                    double *__restrict__ part) {
    const int q = blockIdx.y;
    const BEvent<R> &e = ev[q];
    KSum acc[NQ];
    bulk_accumulate<NC, R>(e.B[cur], e.B[cur ^ 1], e.E, nullptr, nullptr, e.L, acc,
                           (long)blockIdx.x * blockDim.x + threadIdx.x, (long)gridDim.x * blockDim.x);
    int qq;
    KSum v = block_reduce<NQ>(acc, qq);
    if (qq >= 0) {
        double *p = part + (((long)q * BATCH_RED_CHUNKS + blockIdx.x) * NQ + qq) * 2;
        p[0] = v.s;
        p[1] = v.c;
    }
}

__global__ void k_batch_bulk_final(const double *__restrict__ part, int nev, double *__restrict__ out) {
    const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long)nev * NQ) return;
    const int q = (int)(t / NQ), k = (int)(t % NQ);
    KSum v{0.0, 0.0};
    for (int c = 0; c < BATCH_RED_CHUNKS; c++) {
        const double *p = part + (((long)q * BATCH_RED_CHUNKS + c) * NQ + k) * 2;
        ksum_merge(v, KSum{p[0], p[1]});
    }
    out[t] = v.s + v.c;
}

struct Batch {
    int nc = 2, ng = 4, na = 3, prec = OPX_F32, nev = 0, reunit_every = 0, device = 0;
    double dt = 0, g = 1;
    std::vector<Lat> lats;
    std::vector<size_t> offB0, offB1, offE;
    char *store = nullptr;
    size_t store_bytes = 0;
    void *ev_dev = nullptr;  // BEvent<R>[nev]
    int cur = 0;
    long steps = 0;
    cudaStream_t stream = nullptr;
    // schedule
    // cluster 0: the flat schedule (one launch per step, order_dev / bstart_dev,
    // flat_blocks blocks); otherwise persistent clusters (list_dev / begin_dev)
    int cluster = 0, block = 0, nclusters = 0;
    int *list_dev = nullptr, *begin_dev = nullptr;
    int *order_dev = nullptr, *bstart_dev = nullptr;
    int flat_blocks = 0;
    std::map<std::tuple<int, int, long>, cudaGraphExec_t> graphs;  // (nsteps, cur, step phase) -> graph
    double *red_part = nullptr, *red_out = nullptr, *red_host = nullptr;
    std::string err;
    long launches = 0;
    bool int_offsets = true;  // every event's link and E offsets fit in 32 bits
};

}  // namespace opx

using namespace opx;

struct opx_batch {
    Batch b;
};

static size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

template <typename R>
static void upload_events(Batch &b) {
    std::vector<BEvent<R>> h(b.nev);
    for (int q = 0; q < b.nev; q++) {
        h[q].L = b.lats[q];
        h[q].B[0] = (R *)(b.store + b.offB0[q]);
        h[q].B[1] = (R *)(b.store + b.offB1[q]);
        h[q].E = (R *)(b.store + b.offE[q]);
    }
    cudaMemcpy(b.ev_dev, h.data(), sizeof(BEvent<R>) * b.nev, cudaMemcpyHostToDevice);
}

static void drop_graphs(Batch &b) {
    for (auto &kv : b.graphs) cudaGraphExecDestroy(kv.second);
    b.graphs.clear();
}

static void batch_release(Batch &b) {
    drop_graphs(b);
    void *p[] = {b.store, b.ev_dev, b.list_dev, b.begin_dev, b.order_dev, b.bstart_dev, b.red_part, b.red_out};
    for (void *x : p) if (x) cudaFree(x);
    if (b.red_host) cudaFreeHost(b.red_host);
    if (b.stream) cudaStreamDestroy(b.stream);
}

// A lightweight view of one event as a handle, for the conversion launchers.
static Ctx event_view(const Batch &b, int q) {
    Ctx c;
    c.L = b.lats[q];
    c.nc = b.nc;
    c.ng = b.ng;
    c.na = b.na;
    c.na_ref = b.nc == 3 ? 9 : 3;
    c.prec = b.prec;
    c.rsize = b.prec == OPX_F64 ? 8 : 4;
    c.stream = b.stream;
    return c;
}

// Longest-processing-time assignment of events (weight = sites) to clusters.
static void schedule(Batch &b, int nclusters) {
    std::vector<int> order(b.nev);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return b.lats[x].V > b.lats[y].V; });
    std::vector<long> load(nclusters, 0);
    std::vector<std::vector<int>> bins(nclusters);
    for (int q : order) {
        int best = (int)(std::min_element(load.begin(), load.end()) - load.begin());
        bins[best].push_back(q);
        load[best] += b.lats[q].V;
    }
    std::vector<int> list, begin(1, 0);
    for (auto &bin : bins) {
        list.insert(list.end(), bin.begin(), bin.end());
        begin.push_back((int)list.size());
    }
    if (b.list_dev) cudaFree(b.list_dev);
    if (b.begin_dev) cudaFree(b.begin_dev);
    cudaMalloc(&b.list_dev, sizeof(int) * std::max<size_t>(1, list.size()));
    cudaMalloc(&b.begin_dev, sizeof(int) * begin.size());
    cudaMemcpy(b.list_dev, list.data(), sizeof(int) * list.size(), cudaMemcpyHostToDevice);
    cudaMemcpy(b.begin_dev, begin.data(), sizeof(int) * begin.size(), cudaMemcpyHostToDevice);
    b.nclusters = nclusters;
}

// Flat schedule: events in decreasing size, each one's thread units (sites, or
// site pairs for SU(3) FP32) in blocks of b.block.
static void schedule_flat(Batch &b, int block) {
    std::vector<int> order(b.nev);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return b.lats[x].V > b.lats[y].V; });
    const bool paired = b.nc == 3 && b.prec == OPX_F32;
    std::vector<int> bstart(1, 0);
    for (int q : order) {
        const long V = b.lats[q].V, units = paired ? ((V + 63) >> 6) << 5 : V;
        bstart.push_back(bstart.back() + (int)((units + block - 1) / block));
    }
    if (b.order_dev) cudaFree(b.order_dev);
    if (b.bstart_dev) cudaFree(b.bstart_dev);
    cudaMalloc(&b.order_dev, sizeof(int) * order.size());
    cudaMalloc(&b.bstart_dev, sizeof(int) * bstart.size());
    cudaMemcpy(b.order_dev, order.data(), sizeof(int) * order.size(), cudaMemcpyHostToDevice);
    cudaMemcpy(b.bstart_dev, bstart.data(), sizeof(int) * bstart.size(), cudaMemcpyHostToDevice);
    b.flat_blocks = bstart.back();
    b.nclusters = 0;
}

template <int NC, typename R>
static cudaError_t launch_flat(Batch &b, int nsteps, cudaStream_t st) {
    const long step0 = b.reunit_every > 0 ? b.steps % b.reunit_every : 0L;
    const BEvent<R> *ev = (const BEvent<R> *)b.ev_dev;
    const int *order = b.order_dev, *bstart = b.bstart_dev;
    int nev = b.nev;
    for (int k = 0; k < nsteps; k++) {
        const bool reunit = b.reunit_every > 0 && ((step0 + k + 1) % b.reunit_every) == 0;
        int rd = b.cur ^ ((k + 1) & 1);
        void *args[] = {(void *)&ev, (void *)&order, (void *)&bstart, (void *)&nev, (void *)&rd};
        void *kf = b.int_offsets ? (reunit ? flat_kernel<NC, R, int, true>() : flat_kernel<NC, R, int, false>())
                                 : (reunit ? flat_kernel<NC, R, long, true>() : flat_kernel<NC, R, long, false>());
        cudaError_t e = cudaLaunchKernel(kf, dim3(b.flat_blocks), dim3(b.block), args, 0, st);
        b.launches++;
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

template <int NC, typename R>
static cudaError_t launch_persistent(Batch &b, int nsteps, cudaStream_t st) {
    if (b.cluster == 0) return launch_flat<NC, R>(b, nsteps, st);
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(b.nclusters * b.cluster);
    cfg.blockDim = dim3(b.block);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = b.cluster;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    b.launches++;
    const long step0 = b.reunit_every > 0 ? b.steps % b.reunit_every : 0L;
    const BEvent<R> *ev = (const BEvent<R> *)b.ev_dev;
    const int *list = (const int *)b.list_dev, *begin = (const int *)b.begin_dev;
    const int cur = b.cur, re = b.reunit_every;
    void *args[] = {(void *)&ev, (void *)&list, (void *)&begin, (void *)&nsteps, (void *)&cur, (void *)&step0,
                    (void *)&re};
    void *k = b.int_offsets ? persistent_kernel<NC, R, int>() : persistent_kernel<NC, R, long>();
    return cudaLaunchKernelExC(&cfg, k, args);
}

template <int NC, typename R>
static int max_clusters(Batch &b, int cluster, int block) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(cluster * 152);
    cfg.blockDim = dim3(block);
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = cluster;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    int n = 0;
    void *k = b.int_offsets ? persistent_kernel<NC, R, int>() : persistent_kernel<NC, R, long>();
    if (cudaOccupancyMaxActiveClusters(&n, k, &cfg) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return n;
}

static cudaError_t run_dispatch(Batch &b, int nsteps, cudaStream_t st) {
    if (b.nc == 2) return b.prec == OPX_F64 ? launch_persistent<2, double>(b, nsteps, st) : launch_persistent<2, float>(b, nsteps, st);
    return b.prec == OPX_F64 ? launch_persistent<3, double>(b, nsteps, st) : launch_persistent<3, float>(b, nsteps, st);
}

static int occupancy_dispatch(Batch &b, int cluster, int block) {
    if (b.nc == 2) return b.prec == OPX_F64 ? max_clusters<2, double>(b, cluster, block) : max_clusters<2, float>(b, cluster, block);
    return b.prec == OPX_F64 ? max_clusters<3, double>(b, cluster, block) : max_clusters<3, float>(b, cluster, block);
}

static int configure(Batch &b, int cluster, int block) {
    if (cluster == 0) {
        if (b.nc == 3 && b.prec == OPX_F32 && block > 128) return OPX_ERR_UNSUPPORTED;  // the paired kernel's bound
        b.cluster = 0;
        b.block = block;
        schedule_flat(b, block);
        drop_graphs(b);
        return OPX_OK;
    }
    int n = occupancy_dispatch(b, cluster, block);
    if (n <= 0) return OPX_ERR_UNSUPPORTED;
    b.cluster = cluster;
    b.block = block;
    schedule(b, std::min(n, std::max(1, b.nev)));
    drop_graphs(b);
    return OPX_OK;
}

extern "C" {

int opx_batch_create(int ncolors, int nevents, const int *dims, const double *a, double dt, double g,
                     int precision, int reunit_every, int device, opx_batch **out) {
    if (!out || !dims || nevents < 1 || (ncolors != 2 && ncolors != 3) || !(dt > 0) || !(g > 0) ||
        (precision != OPX_F64 && precision != OPX_F32) || reunit_every < 0)
        return OPX_ERR_INVALID;
    *out = nullptr;
    if (cudaSetDevice(device) != cudaSuccess) { cudaGetLastError(); return OPX_ERR_CUDA; }
    opx_batch *h = new opx_batch();
    Batch &b = h->b;
    b.nc = ncolors;
    b.ng = ncolors == 3 ? 18 : 4;
    b.na = ncolors == 3 ? 8 : 3;
    b.prec = precision;
    b.nev = nevents;
    b.dt = dt;
    b.g = g;
    b.reunit_every = reunit_every;
    b.device = device;
    const size_t rs = precision == OPX_F64 ? 8 : 4;
    size_t off = 0;
    for (int q = 0; q < nevents; q++) {
        double aa[3] = {1, 1, 1};
        for (int i = 0; i < 3; i++) {
            if (dims[3 * q + i] < 1) { delete h; return OPX_ERR_INVALID; }
            if (a) aa[i] = a[3 * q + i];
            if (!(aa[i] > 0)) { delete h; return OPX_ERR_INVALID; }
        }
        Lat L = make_lat(dims + 3 * q, aa, dt, g);
        if (L.V * 4 > 2147483647L) { delete h; return OPX_ERR_INVALID; }
        b.lats.push_back(L);
        if (!(link_elems(L.V, b.ng) < (1L << 31) - 64 && 3L * b.na * L.V < (1L << 31))) b.int_offsets = false;
        const size_t nU = (size_t)link_elems(L.V, b.ng) * rs, nE = (size_t)L.V * 3 * b.na * rs;
        b.offB0.push_back(off); off = align256(off + nU);
        b.offB1.push_back(off); off = align256(off + nU);
        b.offE.push_back(off); off = align256(off + nE);
    }
    bool ok = cudaStreamCreateWithFlags(&b.stream, cudaStreamNonBlocking) == cudaSuccess;
    ok = ok && cudaMalloc(&b.store, off) == cudaSuccess;
    b.store_bytes = off;
    const size_t evb = precision == OPX_F64 ? sizeof(BEvent<double>) : sizeof(BEvent<float>);
    ok = ok && cudaMalloc(&b.ev_dev, evb * nevents) == cudaSuccess;
    ok = ok && cudaMalloc(&b.red_part, sizeof(double) * 2 * NQ * BATCH_RED_CHUNKS * nevents) == cudaSuccess;
    ok = ok && cudaMalloc(&b.red_out, sizeof(double) * NQ * nevents) == cudaSuccess;
    ok = ok && cudaMallocHost(&b.red_host, sizeof(double) * NQ * nevents) == cudaSuccess;
    if (!ok) {
        cudaGetLastError();
        batch_release(b);
        delete h;
        return OPX_ERR_NOMEM;
    }
    cudaMemset(b.store, 0, off);
    if (precision == OPX_F64) upload_events<double>(b); else upload_events<float>(b);
    int rc = configure(b, 4, 128);
    if (rc) rc = configure(b, 1, 128);
    if (rc) { batch_release(b); delete h; return rc; }
    *out = h;
    return OPX_OK;
}

void opx_batch_destroy(opx_batch *h) {
    if (!h) return;
    cudaStreamSynchronize(h->b.stream);
    batch_release(h->b);
    delete h;
}

const char *opx_batch_last_error(const opx_batch *h) { return h ? h->b.err.c_str() : "null batch"; }

static int batch_fail(Batch &b, const std::string &m, int code) {
    b.err = m;
    return code;
}

static int batch_sync(Batch &b, const char *where) {
    cudaError_t e = cudaStreamSynchronize(b.stream);
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e != cudaSuccess) return batch_fail(b, std::string(where) + ": " + cudaGetErrorString(e), OPX_ERR_CUDA);
    return OPX_OK;
}

int opx_batch_upload(opx_batch *h, int q, int field, const double *host, size_t count, int layout) {
    if (!h) return OPX_ERR_INVALID;
    Batch &b = h->b;
    if (q < 0 || q >= b.nev || !host || (field != OPX_FIELD_U && field != OPX_FIELD_UNEXT && field != OPX_FIELD_E))
        return batch_fail(b, "opx_batch_upload: invalid event, field or buffer", OPX_ERR_INVALID);
    Ctx c = event_view(b, q);
    const int nah = layout == OPX_LAYOUT_REF ? c.na_ref : c.na;
    const size_t n = field == OPX_FIELD_E ? (size_t)c.L.V * 3 * nah : (size_t)c.L.V * 3 * c.ng;
    if (count != n) return batch_fail(b, "opx_batch_upload: wrong element count", OPX_ERR_INVALID);
    double *tmp = nullptr;
    if (cudaMalloc(&tmp, n * sizeof(double)) != cudaSuccess) { cudaGetLastError(); return batch_fail(b, "opx_batch_upload: out of device memory", OPX_ERR_NOMEM); }
    cudaMemcpyAsync(tmp, host, n * sizeof(double), cudaMemcpyHostToDevice, b.stream);
    if (field == OPX_FIELD_E) launch_alg_from_host(c, tmp, b.store + b.offE[q], 3, layout);
    else launch_links_from_ref(c, tmp, b.store + (((field == OPX_FIELD_U) == (b.cur == 0)) ? b.offB0[q] : b.offB1[q]));
    int rc = batch_sync(b, "opx_batch_upload");
    cudaFree(tmp);
    return rc;
}

int opx_batch_download(opx_batch *h, int q, int field, double *host, size_t count, int layout) {
    if (!h) return OPX_ERR_INVALID;
    Batch &b = h->b;
    if (q < 0 || q >= b.nev || !host || (field != OPX_FIELD_U && field != OPX_FIELD_UNEXT && field != OPX_FIELD_E))
        return batch_fail(b, "opx_batch_download: invalid event, field or buffer", OPX_ERR_INVALID);
    Ctx c = event_view(b, q);
    const int nah = layout == OPX_LAYOUT_REF ? c.na_ref : c.na;
    const size_t n = field == OPX_FIELD_E ? (size_t)c.L.V * 3 * nah : (size_t)c.L.V * 3 * c.ng;
    if (count != n) return batch_fail(b, "opx_batch_download: wrong element count", OPX_ERR_INVALID);
    double *tmp = nullptr;
    if (cudaMalloc(&tmp, n * sizeof(double)) != cudaSuccess) { cudaGetLastError(); return batch_fail(b, "opx_batch_download: out of device memory", OPX_ERR_NOMEM); }
    if (field == OPX_FIELD_E) launch_alg_to_host(c, b.store + b.offE[q], tmp, 3, layout);
    else launch_links_to_ref(c, b.store + (((field == OPX_FIELD_U) == (b.cur == 0)) ? b.offB0[q] : b.offB1[q]), tmp);
    cudaMemcpyAsync(host, tmp, n * sizeof(double), cudaMemcpyDeviceToHost, b.stream);
    int rc = batch_sync(b, "opx_batch_download");
    cudaFree(tmp);
    return rc;
}

int opx_batch_init_random(opx_batch *h, const uint64_t *seeds, double sigma_a, double sigma_e, double tol_g2) {
    if (!h || !seeds) return OPX_ERR_INVALID;
    Batch &b = h->b;
    // one set-up handle per distinct lattice shape, reused for every event of that shape
    std::map<std::vector<double>, opx_ctx *> work;
    int rc = OPX_OK;
    for (int q = 0; q < b.nev && rc == OPX_OK; q++) {
        const Lat &L = b.lats[q];
        std::vector<double> key = {(double)L.n[0], (double)L.n[1], (double)L.n[2], L.a[0], L.a[1], L.a[2]};
        opx_ctx *w = work.count(key) ? work[key] : nullptr;
        if (!w) {
            opx_config cfg = {};
            cfg.ncolors = b.nc;
            for (int i = 0; i < 3; i++) { cfg.dims[i] = L.n[i]; cfg.a[i] = L.a[i]; }
            cfg.dt = b.dt;
            cfg.g = b.g;
            cfg.precision = b.prec;
            cfg.reunit_every = b.reunit_every;
            cfg.device = b.device;
            rc = opx_create(&cfg, &w);
            if (rc) { b.err = opx_last_error(nullptr); break; }
            work[key] = w;
        }
        rc = opx_init_random(w, seeds[q], sigma_a, sigma_e);
        int it = 0;
        double g2 = 0;
        if (!rc && tol_g2 > 0) rc = opx_gauss_project(w, tol_g2, 5000, &it, &g2);
        if (rc) { b.err = opx_last_error(w); break; }
        Ctx &c = ctx_of(w);
        const size_t rs = b.prec == OPX_F64 ? 8 : 4;
        cudaMemcpy(b.store + (b.cur == 0 ? b.offB0[q] : b.offB1[q]), c.U, (size_t)link_elems(L.V, b.ng) * rs, cudaMemcpyDeviceToDevice);
        cudaMemcpy(b.store + b.offE[q], c.E, (size_t)L.V * 3 * b.na * rs, cudaMemcpyDeviceToDevice);
    }
    for (auto &kv : work) opx_destroy(kv.second);
    if (rc) return rc;
    return batch_sync(b, "opx_batch_init_random");
}

int opx_batch_initialize(opx_batch *h) {
    if (!h) return OPX_ERR_INVALID;
    Batch &b = h->b;
    long vmax = 0;
    for (auto &L : b.lats) vmax = std::max(vmax, L.V);
    dim3 grid((unsigned)std::min<long>(grid_for(vmax, 128), 64), b.nev);
    if (b.nc == 2) {
        if (b.prec == OPX_F64) k_batch_links<2, double><<<grid, 128, 0, b.stream>>>((const BEvent<double> *)b.ev_dev, b.nev, b.cur);
        else k_batch_links<2, float><<<grid, 128, 0, b.stream>>>((const BEvent<float> *)b.ev_dev, b.nev, b.cur);
    } else {
        if (b.prec == OPX_F64) k_batch_links<3, double><<<grid, 128, 0, b.stream>>>((const BEvent<double> *)b.ev_dev, b.nev, b.cur);
        else k_batch_links<3, float><<<grid, 128, 0, b.stream>>>((const BEvent<float> *)b.ev_dev, b.nev, b.cur);
    }
    b.launches++;
    return batch_sync(b, "opx_batch_initialize");
}

static int batch_run(Batch &b, int nsteps, int use_graph) {
    if (nsteps <= 0) return OPX_OK;
    cudaError_t e;
    if (use_graph) {
        auto key = std::make_tuple(nsteps, b.cur, b.reunit_every > 0 ? b.steps % b.reunit_every : 0L);
        auto it = b.graphs.find(key);
        if (it == b.graphs.end()) {
            cudaGraph_t g = nullptr;
            cudaGraphExec_t ge = nullptr;
            e = cudaStreamBeginCapture(b.stream, cudaStreamCaptureModeThreadLocal);
            if (e == cudaSuccess) e = run_dispatch(b, nsteps, b.stream);
            cudaError_t e2 = cudaStreamEndCapture(b.stream, &g);
            if (e == cudaSuccess) e = e2;
            if (e == cudaSuccess) e = cudaGraphInstantiate(&ge, g, 0);
            if (g) cudaGraphDestroy(g);
            if (e != cudaSuccess) { cudaGetLastError(); return batch_fail(b, std::string("opx_batch_run: graph capture: ") + cudaGetErrorString(e), OPX_ERR_CUDA); }
            it = b.graphs.emplace(key, ge).first;
        }
        e = cudaGraphLaunch(it->second, b.stream);
        b.launches += b.cluster == 0 ? nsteps : 1;  // the graph's kernel nodes
    } else {
        e = run_dispatch(b, nsteps, b.stream);
    }
    if (e != cudaSuccess) { cudaGetLastError(); return batch_fail(b, std::string("opx_batch_run: ") + cudaGetErrorString(e), OPX_ERR_CUDA); }
    b.cur ^= (nsteps & 1);
    b.steps += nsteps;
    return OPX_OK;
}

int opx_batch_run(opx_batch *h, int nsteps, int use_graph) {
    if (!h || nsteps < 0) return OPX_ERR_INVALID;
    return batch_run(h->b, nsteps, use_graph);
}

int opx_batch_time_run(opx_batch *h, int nsteps, int use_graph, double *ms) {
    if (!h || nsteps < 0 || !ms) return OPX_ERR_INVALID;
    Batch &b = h->b;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, b.stream);
    int rc = batch_run(b, nsteps, use_graph);
    cudaEventRecord(e1, b.stream);
    cudaEventSynchronize(e1);
    float f = 0;
    cudaEventElapsedTime(&f, e0, e1);
    *ms = f;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc) return rc;
    return batch_sync(b, "opx_batch_time_run");
}

int opx_batch_autotune(opx_batch *h, int steps, int *cluster_out, int *block_out) {
    if (!h || steps < 1) return OPX_ERR_INVALID;
    Batch &b = h->b;
    // snapshot the fields: the trial runs advance the events
    char *snap = nullptr;
    if (cudaMalloc(&snap, b.store_bytes) != cudaSuccess) { cudaGetLastError(); return batch_fail(b, "opx_batch_autotune: out of device memory", OPX_ERR_NOMEM); }
    cudaMemcpyAsync(snap, b.store, b.store_bytes, cudaMemcpyDeviceToDevice, b.stream);
    const int cur0 = b.cur;
    const long steps0 = b.steps;
    const int clusters[] = {0, 1, 2, 4, 8};  // 0: the flat schedule
    const int blocks[] = {128, 256};
    double best = 1e300;
    int bc = b.cluster, bb = b.block;
    for (int c : clusters)
        for (int bl : blocks) {
            if (configure(b, c, bl) != OPX_OK) continue;
            double ms = 0;
            if (batch_run(b, 1, 0) != OPX_OK) continue;  // warm-up
            cudaEvent_t e0, e1;
            cudaEventCreate(&e0);
            cudaEventCreate(&e1);
            cudaEventRecord(e0, b.stream);
            int rc = batch_run(b, steps, 0);
            cudaEventRecord(e1, b.stream);
            cudaEventSynchronize(e1);
            float f = 0;
            cudaEventElapsedTime(&f, e0, e1);
            cudaEventDestroy(e0);
            cudaEventDestroy(e1);
            ms = f;
            if (rc == OPX_OK && ms < best) { best = ms; bc = c; bb = bl; }
        }
    cudaMemcpyAsync(b.store, snap, b.store_bytes, cudaMemcpyDeviceToDevice, b.stream);
    cudaStreamSynchronize(b.stream);
    cudaFree(snap);
    b.cur = cur0;
    b.steps = steps0;
    int rc = configure(b, bc, bb);
    if (cluster_out) *cluster_out = b.cluster;
    if (block_out) *block_out = b.block;
    if (rc) return batch_fail(b, "opx_batch_autotune: no launch configuration fits", rc);
    return batch_sync(b, "opx_batch_autotune");
}

int opx_batch_set_schedule(opx_batch *h, int cluster, int block) {
    if (!h || (cluster != 0 && cluster != 1 && cluster != 2 && cluster != 4 && cluster != 8) ||
        (block != 128 && block != 256))
        return OPX_ERR_INVALID;
    Batch &b = h->b;
    const int c0 = b.cluster, b0 = b.block;
    if (configure(b, cluster, block) != OPX_OK) {
        configure(b, c0, b0);
        return batch_fail(b, "opx_batch_set_schedule: that launch configuration does not fit", OPX_ERR_UNSUPPORTED);
    }
    return batch_sync(b, "opx_batch_set_schedule");
}

int opx_batch_reduce(opx_batch *h, opx_observables *out) {
    if (!h || !out) return OPX_ERR_INVALID;
    Batch &b = h->b;
    dim3 grid(BATCH_RED_CHUNKS, b.nev);
    if (b.nc == 2) {
        if (b.prec == OPX_F64) k_batch_bulk<2, double><<<grid, 256, 0, b.stream>>>((const BEvent<double> *)b.ev_dev, b.cur, b.red_part);
        else k_batch_bulk<2, float><<<grid, 256, 0, b.stream>>>((const BEvent<float> *)b.ev_dev, b.cur, b.red_part);
    } else {
        if (b.prec == OPX_F64) k_batch_bulk<3, double><<<grid, 256, 0, b.stream>>>((const BEvent<double> *)b.ev_dev, b.cur, b.red_part);
        else k_batch_bulk<3, float><<<grid, 256, 0, b.stream>>>((const BEvent<float> *)b.ev_dev, b.cur, b.red_part);
    }
    k_batch_bulk_final<<<grid_for((long)b.nev * NQ, 256), 256, 0, b.stream>>>(b.red_part, b.nev, b.red_out);
    b.launches += 2;
    cudaMemcpyAsync(b.red_host, b.red_out, sizeof(double) * NQ * b.nev, cudaMemcpyDeviceToHost, b.stream);
    int rc = batch_sync(b, "opx_batch_reduce");
    if (rc) return rc;
    for (int q = 0; q < b.nev; q++) {
        const double *r = b.red_host + (size_t)q * NQ;
        const double V = (double)b.lats[q].V;
        opx_observables &o = out[q];
        double es[3], bs[3];
        for (int i = 0; i < 3; i++) { es[i] = r[i] / V; bs[i] = r[3 + i] / V; o.e2[i] = es[i]; o.b2[i] = bs[i]; }
        o.px = -es[0] + es[1] + es[2] - bs[0] + bs[1] + bs[2];
        o.py = +es[0] - es[1] + es[2] + bs[0] - bs[1] + bs[2];
        o.pz = +es[0] + es[1] - es[2] + bs[0] + bs[1] - bs[2];
        o.gauss = r[6] / V;
        o.rho2 = 0.0;
        o.e2_total = es[0] + es[1] + es[2];
        o.b2_total = bs[0] + bs[1] + bs[2];
    }
    return OPX_OK;
}

int opx_batch_config(const opx_batch *h, int *cluster, int *block, int *nclusters) {
    if (!h) return OPX_ERR_INVALID;
    if (cluster) *cluster = h->b.cluster;
    if (block) *block = h->b.block;
    if (nclusters) *nclusters = h->b.nclusters;
    return OPX_OK;
}

long opx_batch_kernel_launches(const opx_batch *h) { return h ? h->b.launches : -1; }

}  // extern "C"
