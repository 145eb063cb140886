// Batched ensemble: many independent, uneven-sized instances (each a
// constant-coefficient 7-point problem with its own coefficients, a static
// source field and a constant Dirichlet border -- the Pennes bioheat update
// of examples/MRIDataPBHEqnFDM/MRIDataPBHEqnFDM.hpp:143-169 with scalar
// coefficients) advanced together.
//
// The reference runs one problem per process; its Python drivers
// (examples/MRIDataPBHEqnFDM/startMCMCFit.py) launch whole runs one after
// the other.  Here every time step of the whole ensemble is ONE launch of a
// persistent kernel: grid = SMs x resident CTAs, each CTA pulls work items
// (instance, 32xBY tile, z-chunk) from a device queue (one atomic counter
// per step) and runs them through the same TMA-fed tile code as the plain
// sweep.  The time loop (a memset of the counters and n_steps launches) is
// captured once into a CUDA graph and replayed.  scafes_batch_autotune
// picks the tile variant, the CTAs per SM and the temporal-blocking depth:
// depth 2 advances each instance two steps per pass over its field with
// the plain sweep's depth-2 kernel (star7_tb.cuh), one launch per instance
// and pass, the instances spread over kSideStreams parallel chains of the
// graph.  For comparison,
// scafes_batch_step_looped runs the reference's schedule on the GPU: one
// plain launch per instance per step.
#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <map>
#include <string>
#include <vector>

#include "star7_tile.cuh"

using namespace scafes;

namespace scafes {
void set_last_error(const char* msg);
}

namespace {

constexpr int kZChunk = 32;  // planes per work item
constexpr int kSideStreams = 16;  // parallel launch chains of a depth-2 step

struct BatchInst {
    Layout L;
    long long off_u[2];  // element offsets of the two iterates in the pool
    long long off_f;     // element offset of the source field
    Star7Coeffs c;
    double gconst;       // Dirichlet value the kernels write (0 in deviation form)
    // Deviation form of the FP32-based element types: the device holds
    // u - shift and F + fshift, fshift = shift * (c0 + 2 sum cp - 1) / cf,
    // which is the same update (a constant Dirichlet value g makes
    // u' - g = c0 (u - g) + sum cp (nb - g) + cf (F + g (c0 + 2 sum cp - 1) / cf)).
    // A field near a large constant value then keeps its pair precision
    // for the deviation.  FP64 keeps shift = 0: the reference's arithmetic.
    double shift, fshift;
};

__global__ void k_add_scalar(double* __restrict__ a, size_t n, double v) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        a[i] += v;
}

struct BatchItem {
    int inst;
    short tx, ty;  // tile indices
    short z0, z1;  // planes [z0, z1)
};

// The persistent loop: pull work items until the step's queue is empty.
template <class P, int BY, int R, int NS>
__device__ __forceinline__ void batch_loop(const BatchInst* __restrict__ inst, const CUtensorMap* __restrict__ maps,
                                           int map_stride, const BatchItem* __restrict__ items, int n_items,
                                           typename P::T* __restrict__ pool, int cur, int* __restrict__ counter,
                                           int* __restrict__ status) {
    using T = typename P::T;
    using G = Tile<T, BY, NS, true>;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    T* st = reinterpret_cast<T*>(smem_raw);
    uint64_t* bar = reinterpret_cast<uint64_t*>(smem_raw + (size_t)NS * G::STRIDE * G::ESZ);
    int& s_item = *reinterpret_cast<int*>(bar + NS);  // after the ring (see smem_bytes)
    ring_init<NS>(bar);
    const int tid = threadIdx.y * BX + threadIdx.x;
    uint32_t base = 0;
    for (;;) {
        if (tid == 0) s_item = atomicAdd(counter, 1);
        __syncthreads();
        const int it = s_item;
        __syncthreads();
        if (it >= n_items) break;
        const BatchItem w = items[it];
        const BatchInst& I = inst[w.inst];
        // Coefficients in registers: read through `I`, every store to the
        // pool could alias them and force a reload per node.
        const Star7Coeffs c = I.c;
        TileJob<T> J;
        J.tm = maps + (long long)(3 * w.inst + cur) * map_stride;
        J.tmf = maps + (long long)(3 * w.inst + 2) * map_stride;
        J.un = pool + I.off_u[cur ^ 1];
        J.fa = pool + I.off_f;
        J.fb = nullptr;
        J.ga = nullptr;
        J.gb = nullptr;
        J.gval = P::from_double(I.gconst);
        J.L = I.L;
        J.time_old = J.time_new = J.corr = Split{0.0, 0.f, 0.f};
        J.table = nullptr;
        if (!star7_tile<P, SRC_A, SCAFES_BORDER_DIRICHLET, BY, R, NS, true>(J, c, w.tx * BX, w.ty * BY, w.z0, w.z1, st, bar,
                                                                     base, status))
            break;
    }
}

template <class P, int BY, int R, int NS>
__global__ void __launch_bounds__(BX * (BY / R))
batch_star7(const BatchInst* __restrict__ inst, const CUtensorMap* __restrict__ maps, int map_stride,
            const BatchItem* __restrict__ items, int n_items, typename P::T* __restrict__ pool, int cur,
            int* __restrict__ counter, int* __restrict__ status) {
    batch_loop<P, BY, R, NS>(inst, maps, map_stride, items, n_items, pool, cur, counter, status);
}

// FP64 variant with a register cap: resident warps hide the latency of
// the FP64 pipe and of the integer-pipe neighbour sums.  One row per
// thread: 6 CTAs (40 registers); two rows: 1024 threads' worth of CTAs (64
// registers, 72 bytes spilled); four rows: no cap (a 64-register cap would
// spill the four rows' integer sums, 1.8 KB).  The FP32 policies keep the
// compiler's choice (a cap spills the pair kernels' row pairs and measured
// slower).
template <int R>
constexpr int batch_f64_min_ctas(int threads) {
    return R == 1 ? 1536 / threads : (R >= 4 ? 0 : 1024 / threads);
}
template <int BY, int R, int NS>
__global__ void __launch_bounds__(BX * (BY / R), batch_f64_min_ctas<R>(BX * (BY / R)))
batch_star7_f64(const BatchInst* __restrict__ inst, const CUtensorMap* __restrict__ maps, int map_stride,
                const BatchItem* __restrict__ items, int n_items, double* __restrict__ pool, int cur,
                int* __restrict__ counter, int* __restrict__ status) {
    batch_loop<PolF64, BY, R, NS>(inst, maps, map_stride, items, n_items, pool, cur, counter, status);
}

// The tile ring plus one int for the work-item broadcast.
template <class T, int BY, int NS>
size_t smem_bytes() { return Tile<T, BY, NS, true>::SMEM + 16; }

}  // namespace

struct scafes_batch {
    int precision = SCAFES_PREC_F64;
    size_t esz = 8;
    std::vector<scafes_batch_instance> desc;
    std::vector<BatchInst> hinst;
    BatchInst* dinst = nullptr;
    void* pool = nullptr;
    size_t pool_elems = 0;
    // Tensor maps: [inst][iterate 0, iterate 1, source][tile] on the device
    // and on the host.
    std::vector<CUtensorMap> hmaps;
    CUtensorMap* dmaps = nullptr;
    // Work items per tile variant.
    std::vector<BatchItem> hitems[STAR7_NUM_TILES];
    BatchItem* ditems[STAR7_NUM_TILES] = {};
    int* counters = nullptr;
    int n_counters = 0;
    int* status = nullptr;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    int tile = 1;
    int ctas_per_sm = 0;  // 0 = occupancy limit
    int depth = 1;        // temporal-blocking depth of scafes_batch_step (1 or 2)
    float depth_ms[2] = {-1.f, -1.f};  // the autotuner's best time per depth
    // Depth 2: per instance the TMA maps of both iterates for the depth-2
    // box, the side streams of the capture and their fork/join events.
    std::vector<CUtensorMap> htb;
    cudaStream_t side[kSideStreams] = {};
    cudaEvent_t fork = nullptr, join[kSideStreams] = {};
    int cur = 0;
    int t = 0;
    int launches = 0;
    bool timed = false;
    // Graphs of the time loop, keyed by (n_steps, cur parity, tile, ctas).
    std::map<long long, cudaGraphExec_t> graphs;
    std::string err;
};

namespace {

int bfail(scafes_batch* b, int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    if (b) b->err = buf;
    scafes::set_last_error(buf);
    return code;
}

#define BTRY(b, call)                                                                          \
    do {                                                                                       \
        cudaError_t e_ = (call);                                                               \
        if (e_ != cudaSuccess)                                                                 \
            return bfail(b, SCAFES_ERR_CUDA, "%s: %s (%s:%d)", #call, cudaGetErrorString(e_), \
                         __FILE__, __LINE__);                                                  \
    } while (0)

int num_sms_dev() {
    int dev = 0, n = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    return n > 0 ? n : 1;
}

void clear_graphs(scafes_batch* b) {
    for (auto& kv : b->graphs) cudaGraphExecDestroy(kv.second);
    b->graphs.clear();
}

// Kernel pointer, block shape and dynamic shared memory of (precision, tile).
struct KernelInfo {
    const void* fn;
    dim3 block;
    size_t smem;
};

// The kernel of (policy, tile): the FP64 policy takes the register-capped
// variant.
template <class P, int BY, int R, int NS>
const void* batch_kernel() {
    if constexpr (std::is_same<P, PolF64>::value) return (const void*)batch_star7_f64<BY, R, NS>;
    else return (const void*)batch_star7<P, BY, R, NS>;
}

template <class P>
KernelInfo kinfo_prec(int tile) {
    using T = typename P::T;
    switch (tile) {
        case 0: return {batch_kernel<P, kTiles[0].by, kTiles[0].r, ring_stages(kTiles[0].ns, true)>(), dim3(BX, kTiles[0].by / kTiles[0].r), smem_bytes<T, kTiles[0].by, ring_stages(kTiles[0].ns, true)>()};
        case 1: return {batch_kernel<P, kTiles[1].by, kTiles[1].r, ring_stages(kTiles[1].ns, true)>(), dim3(BX, kTiles[1].by / kTiles[1].r), smem_bytes<T, kTiles[1].by, ring_stages(kTiles[1].ns, true)>()};
        case 2: return {batch_kernel<P, kTiles[2].by, kTiles[2].r, ring_stages(kTiles[2].ns, true)>(), dim3(BX, kTiles[2].by / kTiles[2].r), smem_bytes<T, kTiles[2].by, ring_stages(kTiles[2].ns, true)>()};
        default: return {batch_kernel<P, kTiles[3].by, kTiles[3].r, ring_stages(kTiles[3].ns, true)>(), dim3(BX, kTiles[3].by / kTiles[3].r), smem_bytes<T, kTiles[3].by, ring_stages(kTiles[3].ns, true)>()};
    }
}

KernelInfo kinfo(int precision, int tile) {
    switch (precision) {
        case SCAFES_PREC_F32: return kinfo_prec<PolF32>(tile);
        case SCAFES_PREC_F32X2: return kinfo_prec<PolF32x2>(tile);
        default: return kinfo_prec<PolF64>(tile);
    }
}

int grid_size(scafes_batch* b, const KernelInfo& k) {
    int occ = 0;
    cudaFuncSetAttribute(k.fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)k.smem);
    cudaFuncSetAttribute(k.fn, cudaFuncAttributePreferredSharedMemoryCarveout, cudaSharedmemCarveoutMaxShared);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k.fn, k.block.x * k.block.y, k.smem);
    if (occ < 1) occ = 1;
    int per_sm = b->ctas_per_sm > 0 && b->ctas_per_sm < occ ? b->ctas_per_sm : occ;
    return num_sms_dev() * per_sm;
}

// Enqueues one step of the whole ensemble (one persistent launch).
int enqueue_step(scafes_batch* b, int cur, int* counter) {
    const KernelInfo k = kinfo(b->precision, b->tile);
    const int grid = grid_size(b, k);
    const int n_items = (int)b->hitems[b->tile].size();
    const int map_stride = STAR7_NUM_TILES;
    const CUtensorMap* maps = b->dmaps + b->tile;
    const BatchInst* inst = b->dinst;
    const BatchItem* items = b->ditems[b->tile];
    void* pool = b->pool;
    int* status = b->status;
    void* args[] = {(void*)&inst, (void*)&maps, (void*)&map_stride, (void*)&items, (void*)&n_items,
                    (void*)&pool, (void*)&cur, (void*)&counter, (void*)&status};
    BTRY(b, cudaLaunchKernel(k.fn, dim3(grid), k.block, args, k.smem, b->stream));
    return SCAFES_OK;
}

int ensure_counters(scafes_batch* b, int n) {
    if (n <= b->n_counters) return SCAFES_OK;
    clear_graphs(b);
    cudaFree(b->counters);
    b->counters = nullptr;
    b->n_counters = 0;
    BTRY(b, cudaMalloc(&b->counters, sizeof(int) * (size_t)n));
    b->n_counters = n;
    return SCAFES_OK;
}

int check_status(scafes_batch* b) {
    int st = 0;
    BTRY(b, cudaMemcpyAsync(&st, b->status, sizeof(int), cudaMemcpyDeviceToHost, b->stream));
    BTRY(b, cudaStreamSynchronize(b->stream));
    if (st != 0) {
        cudaMemsetAsync(b->status, 0, sizeof(int), b->stream);
        return bfail(b, SCAFES_ERR_TIMEOUT, "a batch kernel gave up waiting for its TMA loads; results are invalid");
    }
    return SCAFES_OK;
}

// Depth-2 resources, made on first use: the TMA maps of both iterates of
// every instance for the depth-2 box, the side streams and their events.
int ensure_tb(scafes_batch* b) {
    if (!b->htb.empty()) return SCAFES_OK;
    int bw = 0, bh = 0;
    star7_tb_box(b->precision, &bw, &bh);
    std::vector<CUtensorMap> maps(b->hinst.size() * 2);
    for (size_t i = 0; i < b->hinst.size(); ++i) {
        const BatchInst& I = b->hinst[i];
        for (int buf = 0; buf < 2; ++buf) {
            const CUresult r = make_tensor_map_3d(&maps[i * 2 + buf], (char*)b->pool + (size_t)I.off_u[buf] * b->esz,
                                                  (int)b->esz, I.L.nx, I.L.ny, I.L.nz, (size_t)I.L.pitch * b->esz,
                                                  (size_t)I.L.plane * b->esz, bw, bh);
            if (r != CUDA_SUCCESS)
                return bfail(b, SCAFES_ERR_CUDA, "scafes_batch: cuTensorMapEncodeTiled failed (%d)", (int)r);
        }
    }
    for (int k = 0; k < kSideStreams; ++k) {
        if (!b->side[k]) BTRY(b, cudaStreamCreateWithFlags(&b->side[k], cudaStreamNonBlocking));
        if (!b->join[k]) BTRY(b, cudaEventCreateWithFlags(&b->join[k], cudaEventDisableTiming));
    }
    if (!b->fork) BTRY(b, cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming));
    b->htb.swap(maps);
    return SCAFES_OK;
}

// Enqueues n_pairs depth-2 passes of every instance starting from iterate
// `cur`: instance i on side stream i % kSideStreams, forked from and joined
// back into the batch's stream (inside a capture this makes kSideStreams
// independent chains of the graph).
int enqueue_tb(scafes_batch* b, int cur, int n_pairs) {
    BTRY(b, cudaEventRecord(b->fork, b->stream));
    const int ns = std::min<int>(kSideStreams, (int)b->hinst.size());
    for (int k = 0; k < ns; ++k) BTRY(b, cudaStreamWaitEvent(b->side[k], b->fork, 0));
    for (int pass = 0; pass < n_pairs; ++pass) {
        for (int i = 0; i < (int)b->hinst.size(); ++i) {
            const BatchInst& I = b->hinst[i];
            Star7Launch a;
            a.precision = b->precision;
            a.border = SCAFES_BORDER_DIRICHLET;
            a.tile = 0;
            a.L = I.L;
            a.tm_uo = nullptr;
            a.tm_f = nullptr;
            a.tm_tb = &b->htb[(size_t)i * 2 + cur];
            a.table = nullptr;
            a.status = b->status;
            a.uo = (char*)b->pool + (size_t)I.off_u[cur] * b->esz;
            a.un = (char*)b->pool + (size_t)I.off_u[cur ^ 1] * b->esz;
            a.fa = (char*)b->pool + (size_t)I.off_f * b->esz;
            a.fb = nullptr;
            a.ga = nullptr;
            a.gb = nullptr;
            a.gconst = I.gconst;
            a.c = I.c;
            a.time_old = a.time_new = a.time_new2 = a.mirror_corr = 0.0;
            const cudaError_t e = launch_star7_tb(a, b->side[i % ns]);
            if (e != cudaSuccess) return bfail(b, SCAFES_ERR_CUDA, "scafes_batch depth-2 pass: %s", cudaGetErrorString(e));
        }
        cur ^= 1;
    }
    for (int k = 0; k < ns; ++k) {
        BTRY(b, cudaEventRecord(b->join[k], b->side[k]));
        BTRY(b, cudaStreamWaitEvent(b->stream, b->join[k], 0));
    }
    return SCAFES_OK;
}

void build_items(scafes_batch* b) {
    for (int tile = 0; tile < STAR7_NUM_TILES; ++tile) {
        auto& v = b->hitems[tile];
        v.clear();
        const int by = kTiles[tile].by;
        for (int i = 0; i < (int)b->hinst.size(); ++i) {
            const Layout& L = b->hinst[i].L;
            for (int z0 = 0; z0 < L.nz; z0 += kZChunk)
                for (int ty = 0; ty < (L.ny + by - 1) / by; ++ty)
                    for (int tx = 0; tx < (L.nx + BX - 1) / BX; ++tx)
                        v.push_back({i, (short)tx, (short)ty, (short)z0,
                                     (short)(z0 + kZChunk < L.nz ? z0 + kZChunk : L.nz)});
        }
    }
}

}  // namespace

extern "C" int scafes_batch_star7_coeffs(scafes_batch_instance* in, double coeff_a, double rho_c, double perf) {
    if (!in || rho_c == 0.0) return bfail(nullptr, SCAFES_ERR_ARG, "scafes_batch_star7_coeffs: bad arguments");
    double sum = 0.0;
    for (int p = 0; p < 3; ++p) {
        if (in->n_nodes[p] < 2) return bfail(nullptr, SCAFES_ERR_ARG, "scafes_batch_star7_coeffs: n_nodes < 2");
        const double h = (in->coord_last[p] - in->coord_first[p]) / (in->n_nodes[p] - 1);
        in->cp[p] = in->tau * coeff_a / (h * h);
        sum += in->cp[p];
    }
    in->c0 = 1.0 - 2.0 * sum - in->tau * perf;
    in->cf = in->tau * (1.0 / rho_c);
    return SCAFES_OK;
}

extern "C" const char* scafes_batch_last_error(const scafes_batch* b) {
    return b ? b->err.c_str() : "";
}

extern "C" void scafes_batch_destroy(scafes_batch* b) {
    if (!b) return;
    if (b->stream) cudaStreamSynchronize(b->stream);
    clear_graphs(b);
    cudaFree(b->dinst);
    cudaFree(b->pool);
    cudaFree(b->dmaps);
    for (int i = 0; i < STAR7_NUM_TILES; ++i) cudaFree(b->ditems[i]);
    cudaFree(b->counters);
    cudaFree(b->status);
    if (b->ev0) cudaEventDestroy(b->ev0);
    if (b->ev1) cudaEventDestroy(b->ev1);
    for (int k = 0; k < kSideStreams; ++k) {
        if (b->side[k]) cudaStreamDestroy(b->side[k]);
        if (b->join[k]) cudaEventDestroy(b->join[k]);
    }
    if (b->fork) cudaEventDestroy(b->fork);
    if (b->own_stream && b->stream) cudaStreamDestroy(b->stream);
    delete b;
}

extern "C" int scafes_batch_create(const scafes_batch_instance* in, int n_inst, int precision, void* stream,
                                   scafes_batch** out) {
    if (!out || !in || n_inst < 1) return bfail(nullptr, SCAFES_ERR_ARG, "scafes_batch_create: bad arguments");
    *out = nullptr;
    if (precision != SCAFES_PREC_F64 && precision != SCAFES_PREC_F32X2 && precision != SCAFES_PREC_F32)
        return bfail(nullptr, SCAFES_ERR_UNSUPPORTED, "scafes_batch_create: precision %d not supported", precision);
    for (int i = 0; i < n_inst; ++i)
        for (int p = 0; p < 3; ++p)
            if (in[i].n_nodes[p] < 3 || in[i].n_nodes[p] > 32767)
                return bfail(nullptr, SCAFES_ERR_ARG, "scafes_batch_create: instance %d n_nodes[%d]=%d out of [3, 32767]",
                             i, p, in[i].n_nodes[p]);
    scafes_batch* b = new (std::nothrow) scafes_batch();
    if (!b) return bfail(nullptr, SCAFES_ERR_NOMEM, "scafes_batch_create: out of host memory");
    b->precision = precision;
    b->esz = element_size(precision);
    b->desc.assign(in, in + n_inst);
    auto bail = [&](int code) { scafes_batch_destroy(b); return code; };
    cudaError_t e;
    if (stream) {
        b->stream = (cudaStream_t)stream;
    } else if ((e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking)) != cudaSuccess) {
        bfail(nullptr, SCAFES_ERR_CUDA, "scafes_batch_create: %s", cudaGetErrorString(e));
        return bail(SCAFES_ERR_CUDA);
    } else {
        b->own_stream = true;
    }
    // Pool: per instance two iterates and the source field, each padded.
    b->hinst.resize(n_inst);
    size_t total = 0;
    for (int i = 0; i < n_inst; ++i) {
        BatchInst& I = b->hinst[i];
        I.L = make_layout(in[i].n_nodes[0], in[i].n_nodes[1], in[i].n_nodes[2]);
        const size_t sz = (size_t)I.L.size();
        I.off_u[0] = (long long)total; total += sz;
        I.off_u[1] = (long long)total; total += sz;
        I.off_f = (long long)total; total += sz;
        I.c = make_star7_coeffs(in[i].c0, in[i].cp, in[i].cf);
        I.gconst = in[i].g_value;
        I.shift = I.fshift = 0.0;
        const double k = in[i].c0 + 2.0 * (in[i].cp[0] + in[i].cp[1] + in[i].cp[2]) - 1.0;
        if (precision != SCAFES_PREC_F64 && in[i].g_value != 0.0 && (k == 0.0 || in[i].cf != 0.0)) {
            I.shift = in[i].g_value;
            I.fshift = k == 0.0 ? 0.0 : in[i].g_value * k / in[i].cf;
            I.gconst = 0.0;
        }
    }
    b->pool_elems = total;
    if ((e = cudaMalloc(&b->pool, total * b->esz)) != cudaSuccess) {
        bfail(nullptr, SCAFES_ERR_NOMEM, "scafes_batch_create: pool of %zu bytes: %s", total * b->esz, cudaGetErrorString(e));
        return bail(SCAFES_ERR_NOMEM);
    }
    if ((e = cudaMemsetAsync(b->pool, 0, total * b->esz, b->stream)) != cudaSuccess ||
        (e = cudaMalloc(&b->dinst, sizeof(BatchInst) * n_inst)) != cudaSuccess ||
        (e = cudaMemcpyAsync(b->dinst, b->hinst.data(), sizeof(BatchInst) * n_inst, cudaMemcpyHostToDevice,
                             b->stream)) != cudaSuccess ||
        (e = cudaMalloc(&b->status, sizeof(int))) != cudaSuccess ||
        (e = cudaMemsetAsync(b->status, 0, sizeof(int), b->stream)) != cudaSuccess ||
        (e = cudaEventCreate(&b->ev0)) != cudaSuccess || (e = cudaEventCreate(&b->ev1)) != cudaSuccess) {
        bfail(nullptr, SCAFES_ERR_CUDA, "scafes_batch_create: %s", cudaGetErrorString(e));
        return bail(SCAFES_ERR_CUDA);
    }
    // Fields not uploaded read as 0: in deviation form that is -shift for
    // the iterates and fshift for the source.
    {
        size_t most = 0;
        for (const BatchInst& I : b->hinst)
            if (I.shift != 0.0) most = std::max(most, (size_t)I.L.nx * I.L.ny * I.L.nz);
        if (most > 0) {
            double* stage = nullptr;
            e = cudaMalloc(&stage, most * sizeof(double));
            for (size_t i = 0; i < b->hinst.size() && e == cudaSuccess; ++i) {
                const BatchInst& I = b->hinst[i];
                if (I.shift == 0.0) continue;
                const size_t nn = (size_t)I.L.nx * I.L.ny * I.L.nz;
                const double fill[3] = {-I.shift, -I.shift, I.fshift};
                const long long offs[3] = {I.off_u[0], I.off_u[1], I.off_f};
                for (int k = 0; k < 3 && e == cudaSuccess; ++k) {
                    e = cudaMemsetAsync(stage, 0, nn * sizeof(double), b->stream);
                    if (e == cudaSuccess) {
                        k_add_scalar<<<256, 256, 0, b->stream>>>(stage, nn, fill[k]);
                        e = cudaGetLastError();
                    }
                    if (e == cudaSuccess)
                        e = convert_to_device(precision, stage, (char*)b->pool + (size_t)offs[k] * b->esz, I.L,
                                              b->stream);
                }
            }
            if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
            cudaFree(stage);
            if (e != cudaSuccess) {
                bfail(nullptr, SCAFES_ERR_CUDA, "scafes_batch_create: %s", cudaGetErrorString(e));
                return bail(SCAFES_ERR_CUDA);
            }
        }
    }
    // Tensor maps of every instance, field (two iterates with halo boxes,
    // the source with a 32 x BY box) and tile variant.
    b->hmaps.resize((size_t)n_inst * 3 * STAR7_NUM_TILES);
    for (int i = 0; i < n_inst; ++i) {
        const Layout& L = b->hinst[i].L;
        for (int buf = 0; buf < 3; ++buf)
            for (int tile = 0; tile < STAR7_NUM_TILES; ++tile) {
                const long long off = buf < 2 ? b->hinst[i].off_u[buf] : b->hinst[i].off_f;
                char* base = (char*)b->pool + (size_t)off * b->esz;
                const int bw = buf < 2 ? star7_box_width(precision) : BX;
                const int bh = buf < 2 ? star7_box_height(tile) : star7_box_height(tile) - 2;
                CUresult r = make_tensor_map_3d(&b->hmaps[((size_t)i * 3 + buf) * STAR7_NUM_TILES + tile], base,
                                                (int)b->esz, L.nx, L.ny, L.nz, (size_t)L.pitch * b->esz,
                                                (size_t)L.plane * b->esz, bw, bh);
                if (r != CUDA_SUCCESS) {
                    bfail(nullptr, SCAFES_ERR_CUDA, "scafes_batch_create: cuTensorMapEncodeTiled failed (%d)", (int)r);
                    return bail(SCAFES_ERR_CUDA);
                }
            }
    }
    if ((e = cudaMalloc(&b->dmaps, sizeof(CUtensorMap) * b->hmaps.size())) != cudaSuccess ||
        (e = cudaMemcpyAsync(b->dmaps, b->hmaps.data(), sizeof(CUtensorMap) * b->hmaps.size(), cudaMemcpyHostToDevice,
                             b->stream)) != cudaSuccess) {
        bfail(nullptr, SCAFES_ERR_CUDA, "scafes_batch_create: %s", cudaGetErrorString(e));
        return bail(SCAFES_ERR_CUDA);
    }
    build_items(b);
    for (int tile = 0; tile < STAR7_NUM_TILES; ++tile) {
        const size_t bytes = sizeof(BatchItem) * b->hitems[tile].size();
        if ((e = cudaMalloc(&b->ditems[tile], bytes)) != cudaSuccess ||
            (e = cudaMemcpyAsync(b->ditems[tile], b->hitems[tile].data(), bytes, cudaMemcpyHostToDevice, b->stream)) !=
                cudaSuccess) {
            bfail(nullptr, SCAFES_ERR_CUDA, "scafes_batch_create: %s", cudaGetErrorString(e));
            return bail(SCAFES_ERR_CUDA);
        }
    }
    if ((e = cudaStreamSynchronize(b->stream)) != cudaSuccess) {
        bfail(nullptr, SCAFES_ERR_CUDA, "scafes_batch_create: %s", cudaGetErrorString(e));
        return bail(SCAFES_ERR_CUDA);
    }
    *out = b;
    return SCAFES_OK;
}

static int transfer(scafes_batch* b, int i, int field, double* host, size_t n, bool up) {
    if (!b) return bfail(nullptr, SCAFES_ERR_ARG, "scafes_batch transfer: batch is NULL");
    if (i < 0 || i >= (int)b->hinst.size())
        return bfail(b, SCAFES_ERR_ARG, "scafes_batch transfer: instance %d out of range", i);
    if (field != SCAFES_FIELD_U && field != SCAFES_FIELD_F_A)
        return bfail(b, SCAFES_ERR_ARG, "scafes_batch transfer: field %d (only U and F_A)", field);
    const BatchInst& I = b->hinst[i];
    const size_t nn = (size_t)I.L.nx * I.L.ny * I.L.nz;
    if (!host || n != nn) return bfail(b, SCAFES_ERR_ARG, "scafes_batch transfer: expected %zu values, got %zu", nn, n);
    const long long off = field == SCAFES_FIELD_U ? I.off_u[b->cur] : I.off_f;
    char* dev = (char*)b->pool + (size_t)off * b->esz;
    // Stage through the iterate's other buffer region is not allowed (it
    // holds data), so a temporary dense buffer is used.
    double* stage = nullptr;
    BTRY(b, cudaMalloc(&stage, nn * sizeof(double)));
    cudaError_t e;
    // Deviation form (FP32-based types): the iterate is held as u - shift,
    // the source as F + fshift.
    const double add = field == SCAFES_FIELD_U ? -I.shift : I.fshift;
    if (up) {
        e = cudaMemcpyAsync(stage, host, nn * sizeof(double), cudaMemcpyHostToDevice, b->stream);
        if (e == cudaSuccess && add != 0.0) {
            k_add_scalar<<<256, 256, 0, b->stream>>>(stage, nn, add);
            e = cudaGetLastError();
        }
        if (e == cudaSuccess) e = convert_to_device(b->precision, stage, dev, I.L, b->stream);
    } else {
        e = convert_from_device(b->precision, dev, stage, I.L, b->stream);
        if (e == cudaSuccess && add != 0.0) {
            k_add_scalar<<<256, 256, 0, b->stream>>>(stage, nn, -add);
            e = cudaGetLastError();
        }
        if (e == cudaSuccess) e = cudaMemcpyAsync(host, stage, nn * sizeof(double), cudaMemcpyDeviceToHost, b->stream);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
    cudaFree(stage);
    if (e != cudaSuccess) return bfail(b, SCAFES_ERR_CUDA, "scafes_batch transfer: %s", cudaGetErrorString(e));
    if (up && field == SCAFES_FIELD_U) b->t = 0;
    return SCAFES_OK;
}

extern "C" int scafes_batch_upload(scafes_batch* b, int inst, int field, const double* host, size_t n) {
    return transfer(b, inst, field, const_cast<double*>(host), n, true);
}

extern "C" int scafes_batch_download(scafes_batch* b, int inst, int field, double* host, size_t n) {
    int rc = b ? check_status(b) : SCAFES_OK;
    if (rc) return rc;
    return transfer(b, inst, field, host, n, false);
}

extern "C" int scafes_batch_step(scafes_batch* b, int n_steps) {
    if (!b) return bfail(nullptr, SCAFES_ERR_ARG, "scafes_batch_step: batch is NULL");
    if (n_steps < 0) return bfail(b, SCAFES_ERR_ARG, "scafes_batch_step: n_steps < 0");
    if (n_steps == 0) return SCAFES_OK;
    int rc = ensure_counters(b, n_steps);
    if (rc) return rc;
    const KernelInfo k = kinfo(b->precision, b->tile);
    grid_size(b, k);  // sets the smem attribute outside any capture
    // Depth 2: n_steps / 2 passes, an odd last step by the persistent kernel.
    const int pairs = b->depth == 2 ? n_steps / 2 : 0;
    const int singles = n_steps - 2 * pairs;
    if (pairs > 0) {
        if ((rc = ensure_tb(b))) return rc;
        if (launch_star7_tb_prepare(b->precision) != cudaSuccess)
            return bfail(b, SCAFES_ERR_CUDA, "scafes_batch_step: depth-2 kernel attributes");
    }
    const long long key = ((((long long)n_steps * 2 + b->cur) * 2 + (b->depth - 1)) * 8 + b->tile) * 32 +
                          b->ctas_per_sm;
    auto it = b->graphs.find(key);
    if (it == b->graphs.end()) {
        cudaGraph_t g = nullptr;
        cudaGraphExec_t ge = nullptr;
        BTRY(b, cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
        int rc2 = SCAFES_OK;
        cudaError_t e = cudaMemsetAsync(b->counters, 0, sizeof(int) * (size_t)n_steps, b->stream);
        if (e == cudaSuccess && pairs > 0) rc2 = enqueue_tb(b, b->cur, pairs);
        // Each depth-2 pass writes the other iterate: after `pairs` passes
        // the field is in cur ^ (pairs & 1).
        const int after_pairs = b->cur ^ (pairs & 1);
        for (int s = 0; s < singles && e == cudaSuccess && rc2 == SCAFES_OK; ++s)
            rc2 = enqueue_step(b, after_pairs ^ (s & 1), b->counters + s);
        cudaError_t e2 = cudaStreamEndCapture(b->stream, &g);
        if (e != cudaSuccess || rc2 != SCAFES_OK || e2 != cudaSuccess) {
            if (g) cudaGraphDestroy(g);
            return bfail(b, SCAFES_ERR_CUDA, "scafes_batch_step: graph capture failed: %s",
                         cudaGetErrorString(e != cudaSuccess ? e : e2));
        }
        e = cudaGraphInstantiate(&ge, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) return bfail(b, SCAFES_ERR_CUDA, "scafes_batch_step: %s", cudaGetErrorString(e));
        it = b->graphs.emplace(key, ge).first;
    }
    BTRY(b, cudaEventRecord(b->ev0, b->stream));
    BTRY(b, cudaGraphLaunch(it->second, b->stream));
    BTRY(b, cudaEventRecord(b->ev1, b->stream));
    b->cur ^= (pairs + singles) & 1;  // one iterate swap per pass and per single step
    b->t += n_steps;
    b->launches = pairs * (int)b->hinst.size() + singles;
    b->timed = true;
    return SCAFES_OK;
}

extern "C" int scafes_batch_step_looped(scafes_batch* b, int n_steps) {
    if (!b) return bfail(nullptr, SCAFES_ERR_ARG, "scafes_batch_step_looped: batch is NULL");
    if (n_steps < 0) return bfail(b, SCAFES_ERR_ARG, "scafes_batch_step_looped: n_steps < 0");
    BTRY(b, cudaEventRecord(b->ev0, b->stream));
    int launches = 0;
    for (int s = 0; s < n_steps; ++s) {
        for (int i = 0; i < (int)b->hinst.size(); ++i) {
            const BatchInst& I = b->hinst[i];
            Star7Launch a;
            a.precision = b->precision;
            a.border = SCAFES_BORDER_DIRICHLET;
            a.tile = star7_default_tile(I.L, b->precision);
            a.L = I.L;
            a.tm_uo = &b->hmaps[((size_t)i * 3 + b->cur) * STAR7_NUM_TILES + a.tile];
            a.tm_f = &b->hmaps[((size_t)i * 3 + 2) * STAR7_NUM_TILES + a.tile];
            a.table = nullptr;
            a.status = b->status;
            a.uo = (char*)b->pool + (size_t)I.off_u[b->cur] * b->esz;
            a.un = (char*)b->pool + (size_t)I.off_u[b->cur ^ 1] * b->esz;
            a.fa = (char*)b->pool + (size_t)I.off_f * b->esz;
            a.fb = nullptr;
            a.ga = nullptr;
            a.gb = nullptr;
            a.gconst = I.gconst;
            a.c = I.c;
            a.time_old = a.time_new = a.mirror_corr = 0.0;
            cudaError_t e = launch_star7(a, b->stream);
            if (e != cudaSuccess)
                return bfail(b, SCAFES_ERR_CUDA, "scafes_batch_step_looped: %s", cudaGetErrorString(e));
            ++launches;
        }
        b->cur ^= 1;
        b->t += 1;
    }
    BTRY(b, cudaEventRecord(b->ev1, b->stream));
    b->launches = launches;
    b->timed = true;
    return SCAFES_OK;
}

extern "C" int scafes_batch_last_ms(const scafes_batch* b, float* ms) {
    if (!b || !ms) return bfail(nullptr, SCAFES_ERR_ARG, "scafes_batch_last_ms: NULL argument");
    if (!b->timed) return bfail(nullptr, SCAFES_ERR_STATE, "scafes_batch_last_ms: nothing ran yet");
    cudaError_t e = cudaEventSynchronize(b->ev1);
    if (e == cudaSuccess) e = cudaEventElapsedTime(ms, b->ev0, b->ev1);
    if (e != cudaSuccess) return bfail(nullptr, SCAFES_ERR_CUDA, "scafes_batch_last_ms: %s", cudaGetErrorString(e));
    return SCAFES_OK;
}

extern "C" int scafes_batch_info(const scafes_batch* b, int* n_items, int* launches, int* tile, int* ctas_per_sm,
                                 long long* n_nodes) {
    if (!b) return bfail(nullptr, SCAFES_ERR_ARG, "scafes_batch_info: batch is NULL");
    if (n_items) *n_items = (int)b->hitems[b->tile].size();
    if (launches) *launches = b->launches;
    if (tile) *tile = b->tile + 1;
    if (ctas_per_sm) *ctas_per_sm = b->ctas_per_sm;
    if (n_nodes) {
        long long s = 0;
        for (const auto& I : b->hinst) s += (long long)I.L.nx * I.L.ny * I.L.nz;
        *n_nodes = s;
    }
    return SCAFES_OK;
}

extern "C" int scafes_batch_autotune(scafes_batch* b, int n_steps, int* tile_out, int* ctas_out) {
    if (!b) return bfail(nullptr, SCAFES_ERR_ARG, "scafes_batch_autotune: batch is NULL");
    if (n_steps < 1) return bfail(b, SCAFES_ERR_ARG, "scafes_batch_autotune: n_steps < 1");
    // Trial steps run on copies of the iterates, restored afterwards.
    const size_t bytes = b->pool_elems * b->esz;
    void* save = nullptr;
    BTRY(b, cudaMalloc(&save, bytes));
    cudaError_t e = cudaMemcpyAsync(save, b->pool, bytes, cudaMemcpyDeviceToDevice, b->stream);
    const int cur0 = b->cur, t0 = b->t;
    int best_tile = b->tile, best_ctas = b->ctas_per_sm, best_depth = 1, rc = SCAFES_OK;
    float best = -1.f;
    const int ctas_opts[] = {0, 1, 2, 4};
    // Depth 1: every tile x CTAs per SM; then depth 2 (its own kernel, no
    // tile or CTA choice), over an even number of steps for both.
    const int trial = n_steps + (n_steps & 1);
    b->depth = 1;
    for (int tile = 0; tile < STAR7_NUM_TILES && rc == SCAFES_OK && e == cudaSuccess; ++tile) {
        for (int ci = 0; ci < 4 && rc == SCAFES_OK && e == cudaSuccess; ++ci) {
            b->tile = tile;
            b->ctas_per_sm = ctas_opts[ci];
            rc = scafes_batch_step(b, trial);  // first call captures the graph
            if (rc == SCAFES_OK) rc = scafes_batch_step(b, trial);
            float ms = 0.f;
            if (rc == SCAFES_OK) rc = scafes_batch_last_ms(b, &ms);
            if (rc == SCAFES_OK && (best < 0.f || ms < best)) {
                best = ms;
                best_tile = tile;
                best_ctas = ctas_opts[ci];
            }
        }
    }
    b->depth_ms[0] = best;
    b->depth_ms[1] = -1.f;
    if (rc == SCAFES_OK && e == cudaSuccess) {
        b->depth = 2;
        b->tile = best_tile;
        b->ctas_per_sm = best_ctas;
        rc = scafes_batch_step(b, trial);
        if (rc == SCAFES_OK) rc = scafes_batch_step(b, trial);
        float ms = 0.f;
        if (rc == SCAFES_OK) rc = scafes_batch_last_ms(b, &ms);
        if (rc == SCAFES_OK) {
            b->depth_ms[1] = ms;
            if (ms < best) {
                best = ms;
                best_depth = 2;
            }
        }
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(b->pool, save, bytes, cudaMemcpyDeviceToDevice, b->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
    cudaFree(save);
    b->cur = cur0;
    b->t = t0;
    b->tile = best_tile;
    b->ctas_per_sm = best_ctas;
    b->depth = best_depth;
    b->timed = false;
    if (rc != SCAFES_OK) return rc;
    if (e != cudaSuccess) return bfail(b, SCAFES_ERR_CUDA, "scafes_batch_autotune: %s", cudaGetErrorString(e));
    rc = check_status(b);
    if (rc) return rc;
    if (tile_out) *tile_out = best_tile + 1;
    if (ctas_out) *ctas_out = best_ctas;
    return SCAFES_OK;
}

extern "C" int scafes_batch_set_schedule(scafes_batch* b, int tile, int ctas_per_sm) {
    if (!b) return bfail(nullptr, SCAFES_ERR_ARG, "scafes_batch_set_schedule: batch is NULL");
    if (tile < 1 || tile > STAR7_NUM_TILES || ctas_per_sm < 0 || ctas_per_sm > 16)
        return bfail(b, SCAFES_ERR_ARG, "scafes_batch_set_schedule: tile %d / ctas %d out of range", tile, ctas_per_sm);
    b->tile = tile - 1;
    b->ctas_per_sm = ctas_per_sm;
    return SCAFES_OK;
}

extern "C" int scafes_batch_set_temporal_depth(scafes_batch* b, int depth) {
    if (!b) return bfail(nullptr, SCAFES_ERR_ARG, "scafes_batch_set_temporal_depth: batch is NULL");
    if (depth != 1 && depth != 2)
        return bfail(b, SCAFES_ERR_ARG, "scafes_batch_set_temporal_depth: depth %d (1 or 2)", depth);
    b->depth = depth;
    return SCAFES_OK;
}

extern "C" int scafes_batch_temporal_depth(const scafes_batch* b, int* depth, float* ms_depth1, float* ms_depth2) {
    if (!b || !depth) return bfail(nullptr, SCAFES_ERR_ARG, "scafes_batch_temporal_depth: NULL argument");
    *depth = b->depth;
    if (ms_depth1) *ms_depth1 = b->depth_ms[0];
    if (ms_depth2) *ms_depth2 = b->depth_ms[1];
    return SCAFES_OK;
}
