// thoth_gpu.cu — host side of the C ABI declared in include/thoth_gpu.h.
//
// Turns a ThothBookDesc into a flat device plan (time grid constants, the
// time-ordered Brownian-bridge program, path events, product table), uploads it
// in one copy into a per-process device arena, runs the persistent book kernel
// and the fixed-order FP64 reduction, and finalises premium / trust exactly as
// the reference's indicators do (monte_carlo_node.cpp:26-40).
#include "thoth_gpu.h"
#include "engine.cuh"
#include "american.cuh"
#include "calib.cuh"

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <new>
#include <stdexcept>
#include <string>
#include <tuple>
#include <vector>

namespace thoth {
cudaError_t launch_book(const DevPlan& P, int variant, int shape, int grid, size_t smem, cudaStream_t st);
int book_shape_count(int variant);
int book_shape_tile_bits(int variant, int shape);
int book_shape_threads(int variant, int shape);
int book_occupancy(int variant, int shape, size_t smem);
size_t book_smem_bytes(int T, int sobol_dims, int stack_depth, int nfa, int n_slots, int n_groups, int n_last,
                       int few_m = 0);
cudaError_t launch_reduce(const double* acc, int rows, int n_acc, double* out, cudaStream_t st);
cudaError_t launch_sobol_points(const uint32_t* V, int dims, int64_t skip, int64_t n_points, uint32_t* out,
                                cudaStream_t st);
cudaError_t launch_quantile(const uint32_t* x, int64_t n, float* out, cudaStream_t st);
cudaError_t launch_bridge(const DevPlan& P, int grid, size_t smem, float* out, cudaStream_t st);
cudaError_t launch_gather_low(const uint32_t* lo_all, const int* order, int n, int T, uint32_t* out, cudaStream_t st);
cudaError_t launch_gather_low_batch(const uint32_t* lo_all, const void* jobs, int n_books, cudaStream_t st);
cudaError_t launch_reduce_batch(const void* jobs, int n_books, int max_acc, cudaStream_t st);
int batch_threads();
int batch_tile_paths();
int batch_occupancy(size_t smem);
cudaError_t launch_batch_kernel(const DevPlan* plans, const BatchBook* books, int n_books, int n_items, int* next,
                                int grid, size_t smem, cudaStream_t st);
cudaError_t launch_fma_peak(float* out, int blocks, int iters, cudaStream_t st);
cudaError_t launch_mufu_peak(float* out, int blocks, int iters, cudaStream_t st);
cudaError_t launch_tc_gemm_test(const void* A, const void* B, int N, int K, float* D, int* status, cudaStream_t st);
} // namespace thoth

// Joe-Kuo table embedded at build time (generated translation unit)
extern "C" const unsigned char thoth_jk_blob[];
extern "C" const size_t thoth_jk_blob_size;

using namespace thoth;

namespace {

thread_local std::string g_err = "";
std::mutex g_mu;

int fail(int code, const std::string& msg)
{
    g_err = msg;
    return code;
}

#define CUDA_TRY(expr)                                                                                         \
    do {                                                                                                       \
        cudaError_t e_ = (expr);                                                                               \
        if (e_ != cudaSuccess)                                                                                 \
            return fail(e_ == cudaErrorMemoryAllocation ? THOTH_GPU_E_NOMEM : THOTH_GPU_E_CUDA,                \
                        std::string(#expr) + ": " + cudaGetErrorString(e_));                                   \
    } while (0)

// ---------------------------------------------------------------------------
// per-process device state
// ---------------------------------------------------------------------------
struct Device {
    bool ready = false;
    int id = 0;
    int sms = 0;
    std::string name;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    uint32_t* sobol_v = nullptr;    // [4097][32]
    uint32_t* sobol_lo = nullptr;   // [4097][256]
    unsigned char* arena = nullptr;
    size_t arena_size = 0;
    unsigned char* pinned = nullptr; // host staging (plan upload + result download)
    size_t pinned_size = 0;
    int* cancel_host = nullptr;      // host-mapped cancel word
    int* cancel_dev = nullptr;
    float* paths = nullptr;          // stored paths of thoth_gpu_simulate_paths
    size_t paths_size = 0;
    unsigned char* lsm = nullptr;    // Longstaff-Schwartz scratch
    size_t lsm_size = 0;
    unsigned char* calib = nullptr;  // leverage calibration scratch
    size_t calib_size = 0;
};
Device g_dev;

int max_dims() { return 4097; }

// the largest tail table of one book (dimensions beyond the Sobol budget x paths, floats)
constexpr size_t TAIL_MAX_BYTES = size_t(8) << 30;

// direction numbers V[d][32] from the embedded Joe-Kuo table (sobol_generator.cpp:22-76)
bool build_direction_numbers(std::vector<uint32_t>& V)
{
    const unsigned char* b = thoth_jk_blob;
    if (thoth_jk_blob_size < 16 || std::memcmp(b, "JK621201", 8) != 0) return false;
    uint32_t dims, nm;
    std::memcpy(&dims, b + 8, 4);
    std::memcpy(&nm, b + 12, 4);
    const uint32_t* S = reinterpret_cast<const uint32_t*>(b + 16);
    const uint32_t* A = S + dims;
    const uint32_t* MO = A + dims;
    const uint32_t* M = MO + dims + 1;
    const int D = (int)dims + 1;
    V.assign((size_t)D * 32, 0);
    for (int i = 0; i < 32; i++) V[i] = 1u << (31 - i);
    for (int d = 1; d < D; d++) {
        const uint32_t s = S[d - 1], a = A[d - 1];
        const uint32_t* m = M + MO[d - 1];
        uint32_t* v = V.data() + (size_t)d * 32;
        if (s >= 32) {
            for (int i = 0; i < 32; i++) v[i] = m[i] << (31 - i);
        } else {
            for (uint32_t i = 0; i < s; i++) v[i] = m[i] << (31 - i);
            for (uint32_t i = s; i < 32; i++) {
                v[i] = v[i - s] ^ (v[i - s] >> s);
                for (uint32_t k = 1; k < s; k++) v[i] ^= ((a >> (s - 1 - k)) & 1u) * v[i - k];
            }
        }
    }
    return true;
}

// low-bit table of dimensions [0, dims): lo[d][t] = XOR of V[d][j] over the set
// bits j of gray(t) = t ^ (t >> 1), t < 256 (the thread part of a tile's points)
void build_low_table(const std::vector<uint32_t>& V, int dims, std::vector<uint32_t>& lo)
{
    lo.assign((size_t)dims * SOBOL_LO_ROW, 0);
    for (int d = 0; d < dims; d++)
        for (int t = 0; t < SOBOL_LO_ROW; t++) {
            const uint32_t g = (uint32_t)(t ^ (t >> 1));
            uint32_t x = 0;
            for (int j = 0; j < 8; j++)
                if ((g >> j) & 1u) x ^= V[(size_t)d * 32 + j];
            lo[(size_t)d * SOBOL_LO_ROW + t] = x;
        }
}

int ensure_device()
{
    if (g_dev.ready) {
        CUDA_TRY(cudaSetDevice(g_dev.id));
        return THOTH_GPU_OK;
    }
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) return fail(THOTH_GPU_E_NODEVICE, "no CUDA device");
    // the engine binds to the calling thread's current device at its first call (one process
    // per GPU: each rank selects its device before it calls in), and every later call sets it
    int dev = 0;
    CUDA_TRY(cudaGetDevice(&dev));
    cudaDeviceProp p;
    CUDA_TRY(cudaGetDeviceProperties(&p, dev));
    if (!(p.major == 10 && p.minor == 3))
        return fail(THOTH_GPU_E_NODEVICE, std::string("device ") + p.name + " is not sm_103 (built for sm_103a only)");
    g_dev.id = dev;
    CUDA_TRY(cudaSetDevice(dev));
    g_dev.sms = p.multiProcessorCount;
    g_dev.name = p.name;
    CUDA_TRY(cudaStreamCreateWithFlags(&g_dev.stream, cudaStreamNonBlocking));
    CUDA_TRY(cudaEventCreate(&g_dev.ev0));
    CUDA_TRY(cudaEventCreate(&g_dev.ev1));
    std::vector<uint32_t> V, lo;
    if (!build_direction_numbers(V)) return fail(THOTH_GPU_E_INVALID, "embedded Joe-Kuo table is corrupt");
    build_low_table(V, max_dims(), lo);
    CUDA_TRY(cudaMalloc(&g_dev.sobol_v, V.size() * 4));
    CUDA_TRY(cudaMalloc(&g_dev.sobol_lo, lo.size() * 4));
    CUDA_TRY(cudaMemcpy(g_dev.sobol_v, V.data(), V.size() * 4, cudaMemcpyHostToDevice));
    CUDA_TRY(cudaMemcpy(g_dev.sobol_lo, lo.data(), lo.size() * 4, cudaMemcpyHostToDevice));
    CUDA_TRY(cudaHostAlloc(&g_dev.cancel_host, sizeof(int), cudaHostAllocMapped));
    *g_dev.cancel_host = 0;
    CUDA_TRY(cudaHostGetDevicePointer(&g_dev.cancel_dev, g_dev.cancel_host, 0));
    g_dev.ready = true;
    return THOTH_GPU_OK;
}

// Allocation fault injection (a test hook, thoth_gpu_debug_fail_allocations): the next
// g_fail_allocs allocations of the engine's working buffers fail as on a full device.
// Guarded by g_mu like every other engine state.
int g_fail_allocs = 0;

template <class T>
cudaError_t dev_alloc(T** p, size_t bytes)
{
    if (g_fail_allocs > 0) {
        --g_fail_allocs;
        *p = nullptr;
        return cudaErrorMemoryAllocation;
    }
    return cudaMalloc(p, bytes);
}

template <class T>
cudaError_t host_alloc(T** p, size_t bytes)
{
    if (g_fail_allocs > 0) {
        --g_fail_allocs;
        *p = nullptr;
        return cudaErrorMemoryAllocation;
    }
    return cudaHostAlloc(p, bytes, cudaHostAllocDefault);
}

int ensure_arena(size_t bytes)
{
    if (bytes <= g_dev.arena_size) return THOTH_GPU_OK;
    if (g_dev.arena) cudaFree(g_dev.arena);
    g_dev.arena = nullptr;
    g_dev.arena_size = 0;
    const size_t sz = std::max(bytes, (size_t)1 << 22) * 5 / 4;
    CUDA_TRY(dev_alloc(&g_dev.arena, sz));
    g_dev.arena_size = sz;
    return THOTH_GPU_OK;
}

int ensure_paths(size_t bytes)
{
    if (bytes <= g_dev.paths_size) return THOTH_GPU_OK;
    if (g_dev.paths) cudaFree(g_dev.paths);
    g_dev.paths = nullptr;
    g_dev.paths_size = 0;
    CUDA_TRY(dev_alloc(&g_dev.paths, bytes));
    g_dev.paths_size = bytes;
    return THOTH_GPU_OK;
}

int ensure_pinned(size_t bytes)
{
    if (bytes <= g_dev.pinned_size) return THOTH_GPU_OK;
    if (g_dev.pinned) cudaFreeHost(g_dev.pinned);
    g_dev.pinned = nullptr;
    g_dev.pinned_size = 0;
    const size_t sz = std::max(bytes, (size_t)1 << 20) * 5 / 4;
    CUDA_TRY(host_alloc(&g_dev.pinned, sz));
    g_dev.pinned_size = sz;
    return THOTH_GPU_OK;
}

// ---------------------------------------------------------------------------
// packing helper: 16-byte aligned sections of one upload blob
// ---------------------------------------------------------------------------
struct Blob {
    std::vector<unsigned char> bytes;
    template <class T>
    size_t put(const std::vector<T>& v)
    {
        const size_t off = (bytes.size() + 15) & ~size_t(15);
        bytes.resize(off + v.size() * sizeof(T) + 16);
        if (!v.empty()) std::memcpy(bytes.data() + off, v.data(), v.size() * sizeof(T));
        bytes.resize(off + v.size() * sizeof(T));
        return off;
    }
};

// ---------------------------------------------------------------------------
// Brownian bridge: the reference schedule (path_generator.cpp:49-120) and its
// time-ordered program. Processing dates 1..m in order, date i is either a
// pending right anchor (pop) or the end of a chain of nodes whose left anchor
// is date i-1; every node but the last in a chain is pushed.
// ---------------------------------------------------------------------------
struct BridgeProgram {
    std::vector<StepProg> prog;
    std::vector<BridgeNode> nodes;
    int stack_depth = 1;
};

bool build_bridge(const std::vector<double>& t, BridgeProgram& out, std::string& err)
{
    const int m = (int)t.size() - 1;
    std::vector<int> bi(m), li(m), ri(m);
    std::vector<double> lw(m), rw(m), sd(m);
    auto bt = [&](int k) { return t[(size_t)k + 1]; };
    std::vector<int> map(m, 0);
    map[m - 1] = 1;
    bi[0] = m - 1;
    sd[0] = std::sqrt(bt(m - 1));
    lw[0] = rw[0] = 0.0;
    int j = 0;
    for (int i = 1; i < m; i++) {
        while (map[j]) j++;
        int k = j;
        while (!map[k]) k++;
        int l = j + ((k - 1 - j) >> 1);
        map[l] = i + 1;
        bi[i] = l;
        li[i] = j;
        ri[i] = k;
        if (j != 0) {
            lw[i] = (bt(k) - bt(l)) / (bt(k) - bt(j - 1));
            rw[i] = (bt(l) - bt(j - 1)) / (bt(k) - bt(j - 1));
            sd[i] = std::sqrt((bt(l) - bt(j - 1)) * (bt(k) - bt(l)) / (bt(k) - bt(j - 1)));
        } else {
            lw[i] = (bt(k) - bt(l)) / bt(k);
            rw[i] = bt(l) / bt(k);
            sd[i] = std::sqrt(bt(l) * (bt(k) - bt(l)) / bt(k));
        }
        j = k + 1;
        if (j >= m) j = 0;
    }
    // gap (left date, right date) -> build step; point date of each build step
    std::map<std::pair<int, int>, int> gap;
    std::vector<int> point(m);
    for (int i = 0; i < m; i++) {
        point[i] = bi[i] + 1;
        if (i > 0) gap[{li[i], ri[i] + 1}] = i;
    }
    auto node_of = [&](int s) {
        BridgeNode n;
        n.lw = (float)lw[s];
        n.rw = (float)rw[s];
        n.sd = (float)sd[s];
        n.bstep = s;
        return n;
    };
    std::vector<int> stack; // pending dates
    out.prog.assign(m, StepProg{0, 0});
    out.nodes.clear();
    int depth = 0;
    for (int i = 1; i <= m; i++) {
        StepProg sp{(int)out.nodes.size(), 0};
        if (i == 1) {
            out.nodes.push_back(node_of(0));
            sp.count = 1;
            if (m == 1) {
                out.prog[0] = sp;
                continue;
            }
            stack.push_back(m);
        }
        if (stack.back() == i) {
            if (sp.count != 0) {
                err = "bridge program: unexpected pop after push";
                return false;
            }
            stack.pop_back();
            out.prog[i - 1] = sp;
            continue;
        }
        for (;;) {
            const int b = stack.back();
            auto it = gap.find({i - 1, b});
            if (it == gap.end()) {
                err = "bridge program: no node for gap";
                return false;
            }
            out.nodes.push_back(node_of(it->second));
            sp.count++;
            if (point[it->second] == i) break;
            stack.push_back(point[it->second]);
        }
        depth = std::max(depth, (int)stack.size());
        out.prog[i - 1] = sp;
    }
    out.stack_depth = depth + 1;
    return true;
}

// per-step records: first node inline, node count, 1/sqrt(dt), event flag; one zero record
// past the last step, which a load one step ahead reads at the last step
std::vector<StepRec> make_recs(const BridgeProgram& bp, const std::vector<float>& isd, const std::vector<char>& ev_flag,
                               int ref_factors)
{
    const size_t N = isd.size();
    std::vector<StepRec> recs(N + 1);
    std::memset(&recs[N], 0, sizeof(StepRec));
    for (size_t i = 0; i < N; i++) {
        StepRec& r = recs[i];
        std::memset(&r, 0, sizeof r);
        r.isd = isd[i];
        r.ev = ev_flag.empty() ? 0 : ev_flag[i];
        if (i < bp.prog.size()) {
            const StepProg& p = bp.prog[i];
            r.count = p.count;
            r.first = p.first + 1;
            if (p.count > 0) {
                const BridgeNode& n = bp.nodes[p.first];
                r.lw = n.lw;
                r.rw = n.rw;
                r.sd = n.sd;
                r.dim = n.bstep * ref_factors;
            }
        }
    }
    return recs;
}

// Sobol dimensions in the order the step loop consumes them: per step, per node
// of its chain, the active spot factors, then the active variance factors
// (the factor loop of bridge_step); with one pass per asset (per_asset), the
// same for each asset in turn. Dimensions beyond the Sobol budget are left out.
std::vector<int> sobol_order(const BridgeProgram& bp, const DevPlan& D, bool per_asset = false)
{
    std::vector<int> order;
    if (!D.use_sobol) return order;
    const int passes = per_asset ? D.n_assets : 1;
    for (int pass = 0; pass < passes; pass++) {
        const int a_lo = per_asset ? pass : 0, a_hi = per_asset ? pass + 1 : D.n_assets;
        for (const StepProg& sp : bp.prog)
            for (int k = 0; k < sp.count; k++) {
                const int d0 = bp.nodes[sp.first + k].bstep * D.ref_factors;
                for (int a = a_lo; a < a_hi; a++)
                    if (D.cidx_spot[a] >= 0 && d0 + D.fid_spot[a] < D.sobol_dims) order.push_back(d0 + D.fid_spot[a]);
                for (int a = a_lo; a < a_hi; a++)
                    if (D.cidx_var[a] >= 0 && d0 + D.fid_var[a] < D.sobol_dims) order.push_back(d0 + D.fid_var[a]);
            }
    }
    return order;
}

// ---------------------------------------------------------------------------
// autotuned launch choices, keyed by book size: (kernel variant before the
// uniform-step promotion, ceil(log2 paths), ceil(log2 steps)) -> (launch shape,
// CTAs per SM, grid policy); filled by the autotuner or an autotune file
// ---------------------------------------------------------------------------
using TuneKey = std::tuple<int, int, int>;
struct TuneChoice {
    int shape = 0, per_sm = 0, policy = 0;
};
std::map<TuneKey, TuneChoice> g_tuned;

int ceil_log2(int64_t x)
{
    int k = 0;
    while (((int64_t)1 << k) < x && k < 62) k++;
    return k;
}

TuneKey tune_key(int base_variant, int64_t paths, int steps) { return TuneKey(base_variant, ceil_log2(paths), ceil_log2(steps)); }

// ---------------------------------------------------------------------------
// plan
// ---------------------------------------------------------------------------
struct Plan {
    DevPlan dp{};
    Blob blob;
    // offsets of the sections inside the blob
    size_t o_steps, o_isd, o_prog, o_nodes, o_recs, o_evr, o_ev, o_lay, o_map, o_levv, o_ginit, o_prod, o_vterm, o_comp,
        o_sord;
    int variant = 1, base_variant = 1, shape = 0, T = 256;
    size_t smem = 0;
    int n_products = 0;
    int64_t paths = 0;
    std::vector<int> greek_mask;
};

bool finite(double x) { return std::isfinite(x); }

// Untuned shape of a single-asset-kernel plan: (8, 2), unless shared memory
// caps the CTAs per SM so low that (8, 1), with the same tile and twice the
// threads per CTA, keeps more threads resident. Needs a device (else 0).
int default_shape(int variant, size_t smem)
{
    static std::map<std::pair<int, size_t>, int> memo;
    auto key = std::make_pair(variant, smem);
    auto it = memo.find(key);
    if (it != memo.end()) return it->second;
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) {
        cudaGetLastError();
        return 0;
    }
    const int t0 = book_occupancy(variant, 0, smem) * book_shape_threads(variant, 0);
    const int t1 = book_occupancy(variant, 1, smem) * book_shape_threads(variant, 1);
    const int shape = t1 > t0 ? 1 : 0;
    memo[key] = shape;
    return shape;
}

// shape < 0: the autotuned shape for the book's size, else the default
int build_plan(const ThothBookDesc* d, Plan& P, int shape = -1)
{
    const bool untuned = shape < 0;
    if (!d) return fail(THOTH_GPU_E_INVALID, "null descriptor");
    const int nd = d->n_dates, N = nd - 1, NA = d->n_assets;
    if (nd < 2 || nd > THOTH_MAX_DATES) return fail(THOTH_GPU_E_INVALID, "n_dates must be in [2, THOTH_MAX_DATES]");
    if (!d->t) return fail(THOTH_GPU_E_INVALID, "t is null");
    if (NA < 1 || NA > THOTH_MAX_ASSETS || !d->assets)
        return fail(NA > THOTH_MAX_ASSETS ? THOTH_GPU_E_TOO_LARGE : THOTH_GPU_E_INVALID, "n_assets out of range");
    if (d->n_products < 1 || d->n_products > THOTH_MAX_PRODUCTS || !d->products)
        return fail(d->n_products > THOTH_MAX_PRODUCTS ? THOTH_GPU_E_TOO_LARGE : THOTH_GPU_E_INVALID,
                    "n_products out of range");
    if (d->paths <= 1) return fail(THOTH_GPU_E_INVALID, "paths must be > 1");
    if (d->sobol_skip < 0) return fail(THOTH_GPU_E_INVALID, "sobol_skip must be >= 0");
    if (d->use_sobol && (uint64_t)d->sobol_skip + (uint64_t)d->paths >= ((uint64_t)1 << 32))
        return fail(THOTH_GPU_E_TOO_LARGE, "sobol_skip + paths must stay below 2^32 (32-bit direction numbers)");
    // time lists (monte_carlo_node.cpp:100-124)
    std::vector<double> tl(nd), dtl(nd, 0.0);
    for (int i = 0; i < nd; i++) {
        if (d->days) {
            tl[i] = (double)(d->days[i] - d->days[0]) / 365.0;
            if (i > 0) dtl[i] = (double)(d->days[i] - d->days[i - 1]) / 365.0;
        } else {
            tl[i] = d->t[i];
            if (i > 0) dtl[i] = d->t[i] - d->t[i - 1];
        }
        if (!finite(tl[i]) || (i > 0 && !(tl[i] > tl[i - 1])))
            return fail(THOTH_GPU_E_INVALID, "dates must be strictly increasing");
    }
    if (tl[0] != 0.0) return fail(THOTH_GPU_E_INVALID, "t[0] must be 0");

    DevPlan& D = P.dp;
    std::memset(&D, 0, sizeof D);
    D.n_steps = N;
    D.n_assets = NA;
    D.use_sobol = d->use_sobol ? 1 : 0;
    D.greeks = d->greeks & (THOTH_GREEK_DELTA | THOTH_GREEK_VEGA);
    D.skip = d->sobol_skip;
    D.paths = d->paths;
    D.seed = d->seed;
    // factors: spots first, then variance noises (pricer_mcl.cpp:414-432)
    int F = NA, n_stoch = 0, n_lsv = 0;
    bool mixed = false;
    for (int a = 0; a < NA; a++) {
        const ThothAsset& A = d->assets[a];
        if (A.model < THOTH_MODEL_GBM || A.model > THOTH_MODEL_LSV) return fail(THOTH_GPU_E_INVALID, "bad model");
        if (!A.carry) return fail(THOTH_GPU_E_INVALID, "asset carry is null");
        if (!(A.spot > 0) || !finite(A.spot)) return fail(THOTH_GPU_E_INVALID, "spot must be > 0");
        D.model[a] = A.model;
        D.s0[a] = (float)A.spot;
        D.vol[a] = (float)A.vol;
        D.v0[a] = (float)A.v0;
        D.fid_spot[a] = a;
        D.cidx_spot[a] = a;
        D.fid_var[a] = -1;
        D.cidx_var[a] = -1;
        if (A.model != THOTH_MODEL_GBM) {
            D.fid_var[a] = NA + n_stoch;
            D.cidx_var[a] = NA + n_stoch;
            n_stoch++;
            F++;
            if (!(A.kappa > 0) || !(A.v0 >= 0) || !(A.theta >= 0) || !(A.xi >= 0) || !(std::fabs(A.rho) <= 1))
                return fail(THOTH_GPU_E_INVALID, "bad Heston parameters");
            D.degenerate[a] = (A.xi <= 1e-12) ? 1 : 0;
        } else if (!(A.vol >= 0) || !finite(A.vol)) {
            return fail(THOTH_GPU_E_INVALID, "bad GBM vol");
        }
        if (A.model == THOTH_MODEL_LSV) {
            n_lsv++;
            if (A.lev_points < 2 || !A.lev_ln_step || !A.lev_offset || !A.lev_values)
                return fail(THOTH_GPU_E_INVALID, "LSV asset needs leverage layers");
            if (A.lev_points > THOTH_MAX_LEV_POINTS)
                return fail(THOTH_GPU_E_TOO_LARGE, "lev_points above THOTH_MAX_LEV_POINTS");
        }
        if (a > 0 && A.model != d->assets[0].model) mixed = true;
    }
    D.ref_factors = F;
    D.n_factors_active = F;
    D.sobol_dims = d->use_sobol ? (int)std::min<long>((long)N * F, max_dims()) : 0;
    // dimensions beyond the Sobol budget: the reference Rng's stream, drawn into the book's
    // tail table before its kernel (tail_normals)
    D.n_tail = d->use_sobol ? (int)((long)N * F - D.sobol_dims) : 0;
    D.tail_ld = d->paths;
    if (D.n_tail > 0) {
        if ((double)D.n_tail * (double)d->paths * sizeof(float) > (double)TAIL_MAX_BYTES)
            return fail(THOTH_GPU_E_TOO_LARGE, "Gaussians beyond the Sobol budget exceed 8 GiB: fewer paths or dates");
        tail_normals_prepare(); // before any capture; retried (and its error reported) at the launch
        cudaGetLastError();
    }
    D.corr = 0;
    if (NA > 1 && d->cholesky) {
        for (int u = 0; u < NA; u++)
            for (int v = 0; v < NA; v++) {
                const double l = d->cholesky[u * NA + v];
                if (!finite(l)) return fail(THOTH_GPU_E_INVALID, "cholesky not finite");
                D.chol[u * MAX_ASSETS + v] = (float)l;
            }
        D.corr = 1;
        D.corr_all = d->correlate_all_spots ? 1 : 0;
    }
    // variant (tile size fixed by it; uniform-step variants decided below). The
    // reference correlates only GBM spots (correlated_noise_node.cpp:15-27): a
    // multi-asset book without a correlated GBM name has independent assets and
    // runs them one after the other (variant 6), unless the book asks for every
    // spot noise to be correlated (correlate_all_spots).
    bool any_gbm = false;
    for (int a = 0; a < NA; a++) any_gbm |= d->assets[a].model == THOTH_MODEL_GBM;
    if (NA == 1 && !mixed && !D.corr) {
        P.variant = d->assets[0].model; // 0 GBM, 1 Heston, 2 LSV
    } else if (D.corr && (any_gbm || D.corr_all)) {
        P.variant = 3;
    } else {
        P.variant = 6;
    }
    D.stack_factors = P.variant == 6 ? 2 : D.n_factors_active;
    P.base_variant = P.variant;
    bool tuned = false;
    if (shape < 0) {
        auto it = g_tuned.find(tune_key(P.variant, d->paths, N));
        tuned = it != g_tuned.end();
        shape = tuned ? it->second.shape : 0;
    }
    if (shape >= book_shape_count(P.variant)) shape = 0;
    P.shape = shape;
    P.T = 1 << book_shape_tile_bits(P.variant, shape);
    const int T = P.T;
    (void)mixed;

    // bridge program (path-generator times: YearFraction(today, d_i) = tl)
    BridgeProgram bp;
    std::string err;
    if (d->use_sobol) {
        if (!build_bridge(tl, bp, err)) return fail(THOTH_GPU_E_INVALID, err);
    } else {
        bp.prog.assign(N, StepProg{0, 0});
        bp.stack_depth = 0;
    }
    D.stack_depth = bp.stack_depth;
    std::vector<float> isd(N);
    for (int i = 1; i <= N; i++) isd[i - 1] = (float)(1.0 / std::sqrt(tl[i] - tl[i - 1]));

    // per-step asset constants
    std::vector<AssetStep> steps((size_t)N * NA);
    for (int i = 1; i <= N; i++)
        for (int a = 0; a < NA; a++) {
            const ThothAsset& A = d->assets[a];
            AssetStep& s = steps[(size_t)(i - 1) * NA + a];
            std::memset(&s, 0, sizeof s);
            const double dt = dtl[i];
            const double carry_drift = A.carry[i] * tl[i] - A.carry[i - 1] * tl[i - 1];
            if (!finite(carry_drift)) return fail(THOTH_GPU_E_INVALID, "carry not finite");
            if (A.model == THOTH_MODEL_GBM) {
                const double v = A.vol;
                s.c[0] = (float)(carry_drift - v * v / 2 * dt);
                s.c[1] = (float)(v * std::sqrt(dt));
                s.c[2] = (float)std::sqrt(dt);
            } else {
                const double kappa = A.kappa, theta = A.theta, xi = A.xi, rho = A.rho, g = 0.5;
                const double e = std::exp(-kappa * dt);
                s.c[0] = (float)e;
                s.c[1] = (float)(theta * (1 - e));
                s.c[2] = (float)(xi * xi * e / kappa * (1 - e));
                s.c[3] = (float)(theta * xi * xi / (2 * kappa) * (1 - e) * (1 - e));
                s.c[4] = (float)carry_drift;
                if (xi > 1e-12) {
                    s.c[5] = (float)(-rho * kappa * theta / xi * dt);
                    s.c[6] = (float)(g * dt * kappa * rho / xi);
                    s.c[7] = (float)(g * dt * 0.5);
                    s.c[8] = (float)(g * dt * (1.0 - rho * rho));
                    s.c[9] = (float)(rho / xi);
                }
                s.c[10] = (float)dt;
            }
        }

    // uniform steps: every step's constants equal step 1's (bitwise)
    bool uniform = true;
    for (int i = 1; i < N && uniform; i++)
        for (int a = 0; a < NA && uniform; a++)
            if (std::memcmp(&steps[(size_t)i * NA + a], &steps[a], sizeof(AssetStep)) != 0) uniform = false;
    D.uniform_steps = uniform ? 1 : 0;
    if (uniform && P.variant == 1) P.variant = 4;
    if (uniform && P.variant == 0) P.variant = 5;

    // leverage layers, deduplicated per asset
    std::vector<int> lev_layer((size_t)NA * nd, 0);
    std::vector<std::vector<float2>> maps(NA);
    std::vector<std::vector<float>> vals(NA);
    int layers_stride = 1, lev_pts_max = 2;
    for (int a = 0; a < NA; a++) {
        const ThothAsset& A = d->assets[a];
        if (A.model != THOTH_MODEL_LSV) continue;
        D.lev_points[a] = A.lev_points;
        lev_pts_max = std::max(lev_pts_max, A.lev_points);
        std::vector<int> rep; // representative date of each layer
        for (int i = 0; i < nd; i++) {
            int found = -1;
            for (size_t r = 0; r < rep.size() && found < 0; r++) {
                const int k = rep[r];
                if (A.lev_ln_step[k] == A.lev_ln_step[i] && A.lev_offset[k] == A.lev_offset[i] &&
                    std::memcmp(A.lev_values + (size_t)k * A.lev_points, A.lev_values + (size_t)i * A.lev_points,
                                sizeof(double) * A.lev_points) == 0)
                    found = (int)r;
            }
            if (found < 0) {
                if (!(A.lev_ln_step[i] > 0)) return fail(THOTH_GPU_E_INVALID, "lev_ln_step must be > 0");
                found = (int)rep.size();
                rep.push_back(i);
                const double inv = 1.0 / A.lev_ln_step[i];
                maps[a].push_back(make_float2((float)inv, (float)(std::log(A.spot) * inv - (double)A.lev_offset[i])));
                for (int k = 0; k < A.lev_points; k++) vals[a].push_back((float)A.lev_values[(size_t)i * A.lev_points + k]);
            }
            lev_layer[(size_t)a * nd + i] = found;
        }
        layers_stride = std::max(layers_stride, (int)rep.size());
    }
    std::vector<float2> lev_map((size_t)NA * layers_stride, make_float2(0.f, 0.f));
    std::vector<float> lev_values((size_t)NA * layers_stride * lev_pts_max, 0.f);
    for (int a = 0; a < NA; a++) {
        for (size_t r = 0; r < maps[a].size(); r++) lev_map[(size_t)a * layers_stride + r] = maps[a][r];
        const int np = std::max(D.lev_points[a], 1);
        for (size_t r = 0; r < maps[a].size(); r++)
            for (int k = 0; k < D.lev_points[a]; k++)
                lev_values[((size_t)a * layers_stride + r) * lev_pts_max + k] = vals[a][r * np + k];
    }
    D.lev_layers_stride = layers_stride;
    D.lev_row_stride = lev_pts_max; // one row stride for every asset, whatever its point count
    // each LSV step's record carries the leverage layer of the date it ends on (engine.cuh)
    for (int i = 1; i <= N; i++)
        for (int a = 0; a < NA; a++) {
            if (d->assets[a].model != THOTH_MODEL_LSV) continue;
            AssetStep& s = steps[(size_t)(i - 1) * NA + a];
            const int layer = lev_layer[(size_t)a * nd + i];
            const float2 mp = lev_map[(size_t)a * layers_stride + layer];
            const size_t row = ((size_t)a * layers_stride + layer) * lev_pts_max;
            if (row > (size_t)INT32_MAX) return fail(THOTH_GPU_E_TOO_LARGE, "leverage tables too large");
            s.c[12] = mp.x;
            s.c[13] = mp.y;
            const int32_t r32 = (int32_t)row;
            std::memcpy(&s.c[14], &r32, sizeof r32);
        }

    // products -> slots, groups, events
    std::map<std::tuple<int, int, int>, int> slot_of; // (type, asset, date)
    std::map<std::tuple<int, int, double, std::vector<int>>, int> group_of;
    std::vector<float> grp_init;
    std::vector<std::vector<Event>> ev((size_t)nd * NA);
    int n_slots = 0;
    auto slot = [&](int type, int a, int date) {
        auto key = std::make_tuple(type, a, date);
        auto it = slot_of.find(key);
        if (it != slot_of.end()) return it->second;
        const int s = n_slots++;
        slot_of[key] = s;
        Event e{type, s, 0.f, 0};
        ev[(size_t)date * NA + a].push_back(e);
        return s;
    };
    // Running groups shared by products on nested date prefixes: barriers of one
    // asset, direction and quanto shift whose monitor lists are prefixes of one
    // another, and continuous variance sums of one asset and quanto shift, keep
    // one running extreme / sum over the union of their dates; a product that
    // ends before the union reads a snapshot taken at its last date. So a book
    // of barriers with daily monitoring and staggered maturities updates one
    // group per asset and step instead of one per product.
    using RunKey = std::tuple<int, int, double>; // (event type, asset, quanto)
    std::map<RunKey, std::vector<int>> run_dates;
    std::vector<char> run_shared(d->n_products, 0);
    for (int p = 0; p < d->n_products; p++) {
        const ThothProduct& Q = d->products[p];
        if (Q.asset < 0 || Q.asset >= NA || Q.maturity < 0 || Q.maturity > N) continue; // rejected below
        std::vector<int> dates;
        int type;
        if (Q.kind == THOTH_PRODUCT_BARRIER && Q.n_monitor > 0 && Q.monitor) {
            dates.assign(Q.monitor, Q.monitor + Q.n_monitor);
            bool ok = true;
            for (size_t k = 0; k < dates.size(); k++)
                ok = ok && dates[k] >= 0 && dates[k] <= N && (k == 0 || dates[k] >= dates[k - 1]);
            if (!ok) continue;
            type = Q.barrier_up ? EV_GRP_MAX : EV_GRP_MIN;
        } else if (Q.kind == THOTH_PRODUCT_VARIANCE && Q.n_obs <= 0 && Q.maturity >= 1) {
            for (int j = 1; j <= Q.maturity; j++) dates.push_back(j);
            type = EV_GRP_SQ_STEP;
        } else {
            continue;
        }
        std::vector<int>& U = run_dates[RunKey(type, Q.asset, Q.quanto)];
        const size_t L = std::min(U.size(), dates.size());
        if (!std::equal(dates.begin(), dates.begin() + L, U.begin())) continue; // not a prefix: own group
        if (dates.size() > U.size()) U.insert(U.end(), dates.begin() + L, dates.end());
        run_shared[p] = 1;
    }
    std::map<RunKey, int> run_group;
    std::map<std::pair<int, int>, int> snap_of; // (group, date) -> slot
    // the running group of product p (created with its update events on first use)
    auto running = [&](const RunKey& rk, int a, float init) {
        auto it = run_group.find(rk);
        if (it != run_group.end()) return it->second;
        const int g = (int)grp_init.size();
        run_group[rk] = g;
        grp_init.push_back(init);
        const int type = std::get<0>(rk);
        const double q = std::get<2>(rk);
        int prev = 0;
        for (int k : run_dates[rk]) {
            const float pk = (float)(type == EV_GRP_SQ_STEP ? q * (tl[k] - tl[k - 1]) : q * tl[k]);
            ev[(size_t)k * NA + a].push_back(Event{type, g, pk, 0});
            prev = k;
        }
        (void)prev;
        return g;
    };
    // a product's view of running group g at its last date: the group itself when
    // that is the group's last date, else a snapshot slot (taken after the update)
    auto view = [&](const RunKey& rk, int g, int a, int last, DevProduct& R) {
        if (last >= run_dates[rk].back()) {
            R.slot_g = g;
            R.g_snap = 0;
            return;
        }
        auto key = std::make_pair(g, last);
        auto it = snap_of.find(key);
        int sl;
        if (it != snap_of.end()) {
            sl = it->second;
        } else {
            sl = n_slots++;
            snap_of[key] = sl;
            ev[(size_t)last * NA + a].push_back(Event{EV_SNAP_G, sl, 0.f, g});
        }
        R.slot_g = sl;
        R.g_snap = 1;
    };
    const bool want_delta = (D.greeks & THOTH_GREEK_DELTA) != 0, want_vega = (D.greeks & THOTH_GREEK_VEGA) != 0;
    std::vector<DevProduct> prods(d->n_products);
    std::vector<Comp> comps;
    P.greek_mask.assign(d->n_products, 0);
    for (int p = 0; p < d->n_products; p++) {
        const ThothProduct& Q = d->products[p];
        DevProduct& R = prods[p];
        std::memset(&R, 0, sizeof R);
        R.slot_y = R.slot_w = -1;
        if (Q.maturity < 0 || Q.maturity > N) return fail(THOTH_GPU_E_INVALID, "maturity index out of range");
        if (Q.option_type != THOTH_CALL && Q.option_type != THOTH_PUT) return fail(THOTH_GPU_E_INVALID, "bad option type");
        if (!finite(Q.strike) || !finite(Q.zero_rate) || !finite(Q.fx) || !finite(Q.quanto))
            return fail(THOTH_GPU_E_INVALID, "product parameters not finite");
        const int mat = Q.maturity;
        R.kind = Q.kind;
        R.call = Q.option_type == THOTH_CALL;
        R.K = (float)Q.strike;
        R.df = (float)(mat == 0 ? 1.0 : std::exp(tl[0] * Q.zero_rate - tl[mat] * Q.zero_rate));
        R.fx = (float)Q.fx;
        R.qfac = (float)std::exp(-Q.quanto * tl[mat]);
        const bool single = Q.kind != THOTH_PRODUCT_BASKET;
        if (single && (Q.asset < 0 || Q.asset >= NA)) return fail(THOTH_GPU_E_INVALID, "product asset out of range");
        const int a = single ? Q.asset : 0;
        switch (Q.kind) {
        case THOTH_PRODUCT_VANILLA:
        case THOTH_PRODUCT_BARRIER: {
            R.slot_s = slot(EV_SNAP_S, a, mat);
            R.inv_s0 = (float)(1.0 / d->assets[a].spot);
            if (Q.kind == THOTH_PRODUCT_VANILLA) {
                if (want_delta) {
                    P.greek_mask[p] |= 1;
                    if (d->assets[a].model == THOTH_MODEL_LSV) R.slot_y = slot(EV_SNAP_Y, a, mat);
                }
                if (want_vega && d->assets[a].model == THOTH_MODEL_GBM) {
                    P.greek_mask[p] |= 2;
                    R.slot_w = slot(EV_SNAP_W, a, mat);
                    R.vol_t = (float)(d->assets[a].vol * tl[mat]);
                }
            } else {
                if (Q.n_monitor < 0 || (Q.n_monitor > 0 && !Q.monitor)) return fail(THOTH_GPU_E_INVALID, "bad monitor list");
                std::vector<int> mon(Q.monitor, Q.monitor + Q.n_monitor);
                for (size_t k = 0; k < mon.size(); k++)
                    if (mon[k] < 0 || mon[k] > N || (k > 0 && mon[k] < mon[k - 1]))
                        return fail(THOTH_GPU_E_INVALID, "monitor indices must be sorted and in range");
                if (!(Q.barrier_level > 0)) return fail(THOTH_GPU_E_INVALID, "barrier level must be > 0");
                const int type = Q.barrier_up ? EV_GRP_MAX : EV_GRP_MIN;
                if (run_shared[p]) {
                    const RunKey rk(type, a, Q.quanto);
                    view(rk, running(rk, a, Q.barrier_up ? -INFINITY : INFINITY), a, mon.back(), R);
                } else {
                    auto key = std::make_tuple(type, a, Q.quanto, mon);
                    auto it = group_of.find(key);
                    int g;
                    if (it == group_of.end()) {
                        g = (int)grp_init.size();
                        group_of[key] = g;
                        grp_init.push_back(Q.barrier_up ? -INFINITY : INFINITY);
                        for (int k : mon)
                            ev[(size_t)k * NA + a].push_back(Event{type, g, (float)(Q.quanto * tl[k]), 0});
                    } else {
                        g = it->second;
                    }
                    R.slot_g = g;
                }
                R.up = Q.barrier_up ? 1 : 0;
                R.knock_in = Q.barrier_in ? 1 : 0;
                R.level = (float)std::log(Q.barrier_level / d->assets[a].spot);
            }
            break;
        }
        case THOTH_PRODUCT_VARIANCE: {
            std::vector<int> obs;
            if (Q.n_obs > 0) {
                if (!Q.obs) return fail(THOTH_GPU_E_INVALID, "bad observation list");
                obs.assign(Q.obs, Q.obs + Q.n_obs);
                for (size_t k = 0; k < obs.size(); k++)
                    if (obs[k] < 0 || obs[k] > N || (k > 0 && obs[k] <= obs[k - 1]))
                        return fail(THOTH_GPU_E_INVALID, "observation indices must be increasing and in range");
            }
            const int type = obs.empty() ? EV_GRP_SQ_STEP : EV_GRP_SQ_OBS;
            std::vector<int> key_dates = obs.empty() ? std::vector<int>{mat} : obs;
            auto key = std::make_tuple(type, a, Q.quanto, key_dates);
            auto it = group_of.find(key);
            int g = -1;
            if (run_shared[p]) {
                const RunKey rk(type, a, Q.quanto);
                view(rk, running(rk, a, 0.f), a, mat, R);
            } else if (it == group_of.end()) {
                g = (int)grp_init.size();
                group_of[key] = g;
                grp_init.push_back(0.f);
                if (obs.empty()) {
                    for (int j = 1; j <= mat; j++)
                        ev[(size_t)j * NA + a].push_back(Event{type, g, (float)(Q.quanto * (tl[j] - tl[j - 1])), 0});
                } else {
                    int prev = 0;
                    const int row = D.n_last++;
                    for (int o : obs) {
                        ev[(size_t)o * NA + a].push_back(Event{type, g, (float)(Q.quanto * (tl[o] - tl[prev])), row});
                        prev = o;
                    }
                }
            } else {
                g = it->second;
            }
            if (!run_shared[p]) R.slot_g = g;
            const double T = (Q.total_year_fraction > 0) ? Q.total_year_fraction : tl[mat];
            R.inv_T = (float)(T > 0 ? 1.0 / T : 0.0);
            R.past = (float)Q.past_variance;
            R.notional = (float)Q.notional;
            R.kvar = (float)Q.strike_variance;
            break;
        }
        case THOTH_PRODUCT_BASKET: {
            if (Q.n_components < 1 || !Q.components || !Q.weights) return fail(THOTH_GPU_E_INVALID, "basket needs components");
            R.comp_first = (int)comps.size();
            R.comp_n = Q.n_components;
            for (int k = 0; k < Q.n_components; k++) {
                const int c = Q.components[k];
                if (c < 0 || c >= NA || !finite(Q.weights[k])) return fail(THOTH_GPU_E_INVALID, "bad basket component");
                Comp cp;
                cp.slot = slot(EV_SNAP_S, c, mat);
                cp.w = (float)(Q.weights[k] * std::exp(-Q.quanto * tl[mat]));
                cp.slot_y = (want_delta && d->assets[c].model == THOTH_MODEL_LSV) ? slot(EV_SNAP_Y, c, mat) : -1;
                cp.inv_s0 = (float)(1.0 / d->assets[c].spot);
                comps.push_back(cp);
            }
            R.qfac = 1.f;
            if (want_delta) P.greek_mask[p] |= 1;
            break;
        }
        default:
            return fail(THOTH_GPU_E_INVALID, "bad product kind");
        }
        R.greek_mask = P.greek_mask[p];
    }
    if (comps.empty()) comps.push_back(Comp{0, 0.f, -1, 0.f});
    // every product a vanilla and no pathwise Greek: the kernel's lean product loops
    D.vanilla_only = D.greeks == 0;
    for (int p = 0; p < d->n_products; p++) D.vanilla_only &= prods[p].kind == P_VANILLA;
    std::vector<VanTerm> vterms(d->n_products);
    for (int p = 0; p < d->n_products; p++) {
        const DevProduct& R = prods[p];
        const float phi = R.call ? 1.f : -1.f;
        vterms[p] = VanTerm{phi * R.qfac * R.df, -phi * R.K * R.df, R.fx, R.slot_s};
    }
    D.n_slots_used = std::max(n_slots, 1);
    D.n_groups = (int)grp_init.size();
    if (grp_init.empty()) grp_init.push_back(0.f);
    D.n_products = d->n_products;
    // events, ordered per (date, asset)
    std::vector<int2> ev_range((size_t)nd * NA);
    std::vector<Event> events;
    std::vector<char> ev_flag(N, 0);
    for (size_t k = 0; k < ev.size(); k++) {
        ev_range[k] = make_int2((int)events.size(), (int)ev[k].size());
        events.insert(events.end(), ev[k].begin(), ev[k].end());
        const size_t date = k / NA;
        if (!ev[k].empty() && date >= 1) ev_flag[date - 1] = 1;
    }
    if (events.empty()) events.push_back(Event{0, 0, 0.f, 0});
    const std::vector<StepRec> recs = make_recs(bp, isd, ev_flag, F);
    std::vector<int> order = sobol_order(bp, D, P.variant == 6);
    D.n_sobol = (int)order.size();
    if (order.empty()) order.push_back(0);

    // tiles over Sobol indices [skip + 1, skip + paths]
    const int64_t lo = d->sobol_skip + 1, hi = d->sobol_skip + d->paths;
    D.tile_first = lo / T;
    D.n_tiles = hi / T - lo / T + 1;
    // few-product accumulation (kernels.cu, FEW_PRODUCTS): books of at most 4 products whose
    // per-thread moment sums fit in 16 KB of shared memory
    {
        const int few_m = 2 * (1 + (D.greeks ? 3 : 1) * d->n_products);
        D.few_m = (d->n_products <= 4 && (size_t)few_m * T * sizeof(float) <= 16384) ? few_m : 0;
    }
    P.smem = book_smem_bytes(T, D.sobol_dims, D.stack_depth, D.stack_factors, D.n_slots_used, D.n_groups, D.n_last,
                             D.few_m);
    if (P.smem > 227 * 1024) return fail(THOTH_GPU_E_TOO_LARGE, "book needs more shared memory than one SM has");
    D.n_acc = 6 * d->n_products + 2;
    P.n_products = d->n_products;
    P.paths = d->paths;

    // pack
    if (bp.nodes.empty()) bp.nodes.push_back(BridgeNode{0, 0, 0, 0});
    P.o_steps = P.blob.put(steps);
    P.o_isd = P.blob.put(isd);
    P.o_prog = P.blob.put(bp.prog);
    P.o_nodes = P.blob.put(bp.nodes);
    P.o_recs = P.blob.put(recs);
    P.o_evr = P.blob.put(ev_range);
    P.o_ev = P.blob.put(events);
    P.o_lay = P.blob.put(lev_layer);
    P.o_map = P.blob.put(lev_map);
    P.o_levv = P.blob.put(lev_values);
    P.o_ginit = P.blob.put(grp_init);
    P.o_prod = P.blob.put(prods);
    P.o_vterm = P.blob.put(vterms);
    P.o_comp = P.blob.put(comps);
    P.o_sord = P.blob.put(order);
    // shapes 0 and 1 share the 256-path tile, so the plan above serves both
    if (untuned && !tuned && P.variant != 3 && P.shape == 0) P.shape = default_shape(P.variant, P.smem);
    return THOTH_GPU_OK;
}

void bind(Plan& P, unsigned char* base)
{
    DevPlan& D = P.dp;
    D.steps = reinterpret_cast<const AssetStep*>(base + P.o_steps);
    D.inv_sqrt_dt = reinterpret_cast<const float*>(base + P.o_isd);
    D.prog = reinterpret_cast<const StepProg*>(base + P.o_prog);
    D.nodes = reinterpret_cast<const BridgeNode*>(base + P.o_nodes);
    D.recs = reinterpret_cast<const StepRec*>(base + P.o_recs);
    D.ev_range = reinterpret_cast<const int2*>(base + P.o_evr);
    D.events = reinterpret_cast<const Event*>(base + P.o_ev);
    D.lev_layer = reinterpret_cast<const int*>(base + P.o_lay);
    D.lev_map = reinterpret_cast<const float2*>(base + P.o_map);
    D.lev_values = reinterpret_cast<const float*>(base + P.o_levv);
    D.grp_init = reinterpret_cast<const float*>(base + P.o_ginit);
    D.products = reinterpret_cast<const DevProduct*>(base + P.o_prod);
    D.vterms = reinterpret_cast<const VanTerm*>(base + P.o_vterm);
    D.comps = reinterpret_cast<const Comp*>(base + P.o_comp);
    D.sobol_order = reinterpret_cast<const int*>(base + P.o_sord);
    D.sobol_v = g_dev.sobol_v;
    D.sobol_lo = nullptr; // the book's own table: placed by the caller (low_bytes)
    D.cancel = g_dev.cancel_dev;
}

// resident CTAs per SM of a plan's kernel (cached per variant, shape and shared-memory size)
int occupancy_of(const Plan& P)
{
    static std::map<std::tuple<int, int, size_t>, int> occ;
    auto key = std::make_tuple(P.variant, P.shape, P.smem);
    auto it = occ.find(key);
    if (it != occ.end()) return it->second;
    const int per_sm = book_occupancy(P.variant, P.shape, P.smem);
    occ[key] = per_sm;
    return per_sm;
}

// grid policies of the persistent book kernel:
//   0 full      resident CTAs per SM x SMs, capped by the tile count
//   1 balanced  the same number of waves as `full` spread over the fewest CTAs
//   2 half      half the resident CTAs (leaves room for concurrent books)
int grid_policy(int64_t tiles, int64_t full, int policy)
{
    full = std::max<int64_t>(full, 1);
    int64_t g = std::min(full, tiles);
    if (policy == 1) {
        const int64_t waves = (tiles + full - 1) / full;
        g = (tiles + waves - 1) / waves;
    } else if (policy == 2) {
        g = std::min(std::max<int64_t>(full / 2, 1), tiles);
    }
    return (int)std::max<int64_t>(g, 1);
}

// persistent grid of a plan: the autotuned choice for the book's size when the
// plan runs in the tuned shape and no other policy is asked for, else `policy`
int grid_for(const Plan& P, int policy = 0)
{
    const int per_sm = occupancy_of(P);
    if (policy == 0) {
        auto it = g_tuned.find(tune_key(P.base_variant, P.paths, P.dp.n_steps));
        if (it != g_tuned.end() && it->second.shape == P.shape) {
            const int k = it->second.per_sm > 0 ? std::min(it->second.per_sm, per_sm) : per_sm;
            return grid_policy(P.dp.n_tiles, (int64_t)k * g_dev.sms, it->second.policy);
        }
    }
    return grid_policy(P.dp.n_tiles, (int64_t)per_sm * g_dev.sms, policy);
}

double trust_of(double s1, double s2, double n)
{
    double var = (s2 - s1 * s1 / n) / (n - 1);
    if (var < 0) var = 0; // round-off on a constant payoff
    return std::sqrt(var / n);
}

// bytes of a book's low Sobol words in consumption order ([n_sobol][T])
// the book's low words in consumption order, and two rows of padding that the kernel's
// load two entries ahead may read past the last entry
// a book's own device tables after its plan blob: its low Sobol words in consumption order, then
// (aligned) its tail Gaussians
size_t low_words_bytes(const Plan& P) { return sizeof(uint32_t) * ((size_t)P.dp.n_sobol + 2) * P.T; }
size_t low_bytes(const Plan& P)
{
    const size_t lo = low_words_bytes(P);
    if (P.dp.n_tail <= 0) return lo;
    return ((lo + 255) & ~size_t(255)) + sizeof(float) * (size_t)P.dp.n_tail * (size_t)P.dp.tail_ld;
}

// places those tables at lo (a region of low_bytes(P) bytes)
void bind_low(Plan& P, unsigned char* lo)
{
    P.dp.sobol_lo = reinterpret_cast<const uint32_t*>(lo);
    P.dp.tail = P.dp.n_tail > 0 ? reinterpret_cast<const float*>(lo + ((low_words_bytes(P) + 255) & ~size_t(255)))
                                : nullptr;
}

// the book's tail Gaussians (dimensions beyond the Sobol budget) into its tail table
cudaError_t tail_normals(const Plan& P, cudaStream_t st)
{
    cudaError_t e = tail_normals_prepare();
    if (e != cudaSuccess) return e;
    return launch_tail_normals(P.dp.seed, P.dp.n_tail, P.dp.tail_ld, const_cast<float*>(P.dp.tail), st);
}

// the book's low words from the device-wide table (one small gather kernel)
cudaError_t gather_low(const Plan& P, cudaStream_t st)
{
    cudaError_t e = launch_gather_low(g_dev.sobol_lo, P.dp.sobol_order, P.dp.n_sobol, P.T,
                                      const_cast<uint32_t*>(P.dp.sobol_lo), st);
    if (e == cudaSuccess && P.dp.n_tail > 0) e = tail_normals(P, st);
    return e;
}

// device layout of one priced book: [plan blob][low Sobol words][acc rows][out][status]
struct Layout {
    size_t o_lo, o_acc, o_out, o_st, total;
};

Layout layout_of(const Plan& P, int grid)
{
    Layout L;
    const size_t n_acc = (size_t)P.dp.n_acc;
    L.o_lo = (P.blob.bytes.size() + 255) & ~size_t(255);
    L.o_acc = L.o_lo + ((low_bytes(P) + 255) & ~size_t(255));
    L.o_out = L.o_acc + ((sizeof(double) * grid * n_acc + 255) & ~size_t(255));
    L.o_st = L.o_out + ((sizeof(double) * n_acc + 255) & ~size_t(255));
    L.total = L.o_st + 256;
    return L;
}

// launch the book kernel and the reduction on a plan already bound to `base`,
// copy the sums back and finalise the indicators
int run_bound(Plan& P, unsigned char* base, const Layout& L, int grid, ThothBookResult* out, bool gather)
{
    const size_t n_acc = (size_t)P.dp.n_acc;
    cudaStream_t st = g_dev.stream;
    int rc = ensure_pinned(sizeof(double) * n_acc + sizeof(int));
    if (rc) return rc;
    bind_low(P, base + L.o_lo);
    P.dp.acc = reinterpret_cast<double*>(base + L.o_acc);
    P.dp.status = reinterpret_cast<int*>(base + L.o_st);
    CUDA_TRY(cudaMemsetAsync(base + L.o_st, 0, sizeof(int), st));
    CUDA_TRY(cudaEventRecord(g_dev.ev0, st));
    if (gather) CUDA_TRY(gather_low(P, st));
    CUDA_TRY(launch_book(P.dp, P.variant, P.shape, grid, P.smem, st));
    CUDA_TRY(launch_reduce(P.dp.acc, grid, (int)n_acc, reinterpret_cast<double*>(base + L.o_out), st));
    CUDA_TRY(cudaEventRecord(g_dev.ev1, st));
    CUDA_TRY(cudaMemcpyAsync(g_dev.pinned, base + L.o_out, sizeof(double) * n_acc, cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaMemcpyAsync(g_dev.pinned + sizeof(double) * n_acc, base + L.o_st, sizeof(int), cudaMemcpyDeviceToHost,
                             st));
    CUDA_TRY(cudaStreamSynchronize(st));
    float ms = 0;
    CUDA_TRY(cudaEventElapsedTime(&ms, g_dev.ev0, g_dev.ev1));
    int status;
    std::memcpy(&status, g_dev.pinned + sizeof(double) * n_acc, sizeof(int));
    if (status == 1) return fail(THOTH_GPU_E_CANCELLED, "pricing cancelled");
    const double* o = reinterpret_cast<const double*>(g_dev.pinned);
    const double n = (double)P.paths;
    const double nan = std::nan("");
    for (int p = 0; p < P.n_products; p++) {
        const double* a = o + 6 * (size_t)p;
        if (out->premium) out->premium[p] = a[0] / n;
        if (out->trust) out->trust[p] = trust_of(a[0], a[1], n);
        const bool dok = (P.greek_mask[p] & 1) != 0, vok = (P.greek_mask[p] & 2) != 0;
        if (out->delta) out->delta[p] = dok ? a[2] / n : nan;
        if (out->delta_trust) out->delta_trust[p] = dok ? trust_of(a[2], a[3], n) : nan;
        if (out->vega) out->vega[p] = vok ? a[4] / n : nan;
        if (out->vega_trust) out->vega_trust[p] = vok ? trust_of(a[4], a[5], n) : nan;
    }
    out->book_premium = o[6 * (size_t)P.n_products] / n;
    out->book_trust = trust_of(o[6 * (size_t)P.n_products], o[6 * (size_t)P.n_products + 1], n);
    out->device_ms = ms;
    out->h2d_bytes = 0;
    out->d2h_bytes = (int64_t)(sizeof(double) * n_acc + sizeof(int));
    return THOTH_GPU_OK;
}

int price_locked(const ThothBookDesc* book, ThothBookResult* out)
{
    if (!out) return fail(THOTH_GPU_E_INVALID, "null result");
    int rc = ensure_device();
    if (rc) return rc;
    Plan P;
    rc = build_plan(book, P);
    if (rc) return rc;
    const int grid = grid_for(P);
    const Layout L = layout_of(P, grid);
    rc = ensure_arena(L.total);
    if (rc) return rc;
    rc = ensure_pinned(P.blob.bytes.size());
    if (rc) return rc;
    std::memcpy(g_dev.pinned, P.blob.bytes.data(), P.blob.bytes.size());
    CUDA_TRY(cudaMemcpyAsync(g_dev.arena, g_dev.pinned, P.blob.bytes.size(), cudaMemcpyHostToDevice, g_dev.stream));
    bind(P, g_dev.arena);
    rc = run_bound(P, g_dev.arena, L, grid, out, true);
    if (rc) return rc;
    out->h2d_bytes = (int64_t)P.blob.bytes.size();
    return THOTH_GPU_OK;
}

// the book priced as by price_locked, with the spot of one asset stored at every
// date of every path (date-major on the device, copied to the caller's array)
// simulate the book and keep the spot of `asset` at every date of every path in
// g_dev.paths, date-major ([n_steps + 1][paths])
int simulate_device_locked(const ThothBookDesc* book, int asset, Plan& P, double* device_ms)
{
    int rc = ensure_device();
    if (rc) return rc;
    rc = build_plan(book, P);
    if (rc) return rc;
    if (asset < 0 || asset >= P.dp.n_assets) return fail(THOTH_GPU_E_INVALID, "asset out of range");
    const size_t bytes = sizeof(float) * (size_t)(P.dp.n_steps + 1) * (size_t)P.paths;
    const int grid = grid_for(P);
    const Layout L = layout_of(P, grid);
    rc = ensure_arena(L.total);
    if (rc) return rc;
    rc = ensure_paths(bytes);
    if (rc) return rc;
    rc = ensure_pinned(P.blob.bytes.size());
    if (rc) return rc;
    std::memcpy(g_dev.pinned, P.blob.bytes.data(), P.blob.bytes.size());
    CUDA_TRY(cudaMemcpyAsync(g_dev.arena, g_dev.pinned, P.blob.bytes.size(), cudaMemcpyHostToDevice, g_dev.stream));
    bind(P, g_dev.arena);
    P.dp.path_out = g_dev.paths;
    P.dp.path_ld = P.paths;
    P.dp.path_asset = asset;
    ThothBookResult sums;
    std::memset(&sums, 0, sizeof sums);
    rc = run_bound(P, g_dev.arena, L, grid, &sums, true);
    if (rc) return rc;
    if (device_ms) *device_ms = sums.device_ms;
    return THOTH_GPU_OK;
}

int simulate_paths_locked(const ThothBookDesc* book, int asset, float* out, double* device_ms)
{
    if (!out) return fail(THOTH_GPU_E_INVALID, "null output");
    Plan P;
    int rc = simulate_device_locked(book, asset, P, device_ms);
    if (rc) return rc;
    const size_t bytes = sizeof(float) * (size_t)(P.dp.n_steps + 1) * (size_t)P.paths;
    CUDA_TRY(cudaMemcpy(out, g_dev.paths, bytes, cudaMemcpyDeviceToHost));
    return THOTH_GPU_OK;
}

int ensure_lsm(size_t bytes)
{
    if (bytes <= g_dev.lsm_size) return THOTH_GPU_OK;
    if (g_dev.lsm) cudaFree(g_dev.lsm);
    g_dev.lsm = nullptr;
    g_dev.lsm_size = 0;
    CUDA_TRY(dev_alloc(&g_dev.lsm, bytes));
    g_dev.lsm_size = bytes;
    return THOTH_GPU_OK;
}

size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

// float bits t such that (double) S > K <=> bits(S) >= t for a call, (double) S < K <=>
// bits(S) <= t for a put, for every non-negative float S (their bit patterns are ordered
// like their values): the smallest float above K, resp. the largest below it
int32_t itm_threshold(double K, bool call)
{
    float f = (float)K;
    if (call) {
        if (!(K >= 0.0)) return 0;
        if ((double)f <= K) f = std::nextafter(f, INFINITY);
    } else {
        if (!(K > 0.0)) return -1;
        if ((double)f >= K) f = std::nextafter(f, 0.0f);
    }
    int32_t b;
    std::memcpy(&b, &f, sizeof b);
    return b;
}

// One Longstaff-Schwartz pass (american.cu) on the stored paths of io.asset: simulate the
// book, then fit a policy and value it on the same paths, or value the given policy.
int lsm_check(const Plan& P, const LsmPass& io)
{
    const int M = io.M;
    if (M < 2 || M > P.dp.n_steps + 1) return fail(THOTH_GPU_E_INVALID, "exercise grid outside the book's dates");
    if (!(io.norm > 0.0) || !std::isfinite(io.norm) || !std::isfinite(io.strike))
        return fail(THOTH_GPU_E_INVALID, "exercise fit needs a finite strike and a positive moneyness normaliser");
    if ((int)io.df.size() != M || (int)io.disc.size() != M)
        return fail(THOTH_GPU_E_INVALID, "discount arrays must have one entry per exercise date");
    if (!io.fit && ((int)io.beta.size() != 3 * M || (int)io.fit_at.size() != M))
        return fail(THOTH_GPU_E_INVALID, "frozen policy does not match the exercise grid");
    if (P.paths >= ((int64_t)1 << 27)) return fail(THOTH_GPU_E_TOO_LARGE, "American exercise needs fewer than 2^27 paths");
    return THOTH_GPU_OK;
}

int lsm_status(int status)
{
    if (status == 2) return fail(THOTH_GPU_E_CUDA, "exercise fit: a wait timed out");
    if (status == 3) return fail(THOTH_GPU_E_INVALID, "exercise fit: a cashflow or moneyness power is out of range (>= 2^36)");
    if (status != 0) return fail(THOTH_GPU_E_CUDA, "exercise fit: kernel status " + std::to_string(status));
    return THOTH_GPU_OK;
}

// the table block of one contract: df [M], disc [M], beta [3M], fit [M] (int)
size_t lsm_tab_bytes(int M) { return sizeof(double) * 5 * (size_t)M + sizeof(int32_t) * (size_t)M; }

void lsm_fill_tab(unsigned char* h, const LsmPass& io)
{
    const int M = io.M;
    std::memcpy(h, io.df.data(), sizeof(double) * M);
    std::memcpy(h + sizeof(double) * M, io.disc.data(), sizeof(double) * M);
    if (io.fit) {
        std::memset(h + sizeof(double) * 2 * M, 0, sizeof(double) * 3 * M + sizeof(int32_t) * M);
    } else {
        std::memcpy(h + sizeof(double) * 2 * M, io.beta.data(), sizeof(double) * 3 * M);
        std::memcpy(h + sizeof(double) * 5 * M, io.fit_at.data(), sizeof(int32_t) * M);
    }
}

// the exact result sums of `grid` CTA rows
void lsm_results(const Fx128* a, int grid, LsmPass& io)
{
    Fx128 tot[LSM_NACC] = {};
    for (int c = 0; c < grid; c++)
        for (int k = 0; k < LSM_NACC; k++) fx_add(tot[k], a[(size_t)c * LSM_NACC + k]);
    io.sum = fx_to_double(tot[0]);
    io.sum2 = fx_to_double(tot[1]);
    io.euro = fx_to_double(tot[2]);
}

// value a frozen policy on the stored paths (lsm_apply_kernel)
int lsm_apply_locked(const Plan& P, double sim_ms, LsmPass& io)
{
    int rc = lsm_check(P, io);
    if (rc) return rc;
    const int M = io.M;
    const int64_t N = P.paths;
    const int grid = (int)std::max<int64_t>(1, std::min<int64_t>((N + LSM_THREADS - 1) / LSM_THREADS,
                                                                 (int64_t)8 * g_dev.sms));
    const size_t tab = lsm_tab_bytes(M);
    const size_t o_tab = 0, o_scr = align256(tab), scr_bytes = sizeof(float4) * (size_t)M;
    const size_t o_acc = o_scr + align256(scr_bytes);
    const size_t acc_bytes = sizeof(Fx128) * (size_t)grid * LSM_NACC;
    const size_t o_ctl = o_acc + align256(acc_bytes);
    rc = ensure_lsm(o_ctl + 256);
    if (rc) return rc;
    rc = ensure_pinned(std::max(o_scr + scr_bytes, acc_bytes + 2 * sizeof(int) + sizeof(float)));
    if (rc) return rc;
    unsigned char* base = g_dev.lsm;
    unsigned char* h = g_dev.pinned;
    lsm_fill_tab(h, io);
    // the single-precision screen of each date: b0, b1, b2 rounded to float, and 1 where the
    // date has a regression (lsm_apply_kernel)
    float4* scr = reinterpret_cast<float4*>(h + o_scr);
    for (int t = 0; t < M; t++)
        scr[t] = io.fit_at[t] ? make_float4((float)io.beta[3 * (size_t)t], (float)io.beta[3 * (size_t)t + 1],
                                            (float)io.beta[3 * (size_t)t + 2], 1.0f)
                              : make_float4(0.f, 0.f, 0.f, 0.f);
    cudaStream_t st = g_dev.stream;
    CUDA_TRY(cudaMemcpyAsync(base + o_tab, h, o_scr + scr_bytes, cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaMemsetAsync(base + o_ctl, 0, sizeof(int), st));
    LsmArgs A;
    A.S = g_dev.paths;
    A.ld = P.paths;
    A.n = N;
    A.M = M;
    A.call = io.call;
    A.strike = io.strike;
    A.norm = io.norm;
    A.inv_norm = 1.0 / io.norm;
    A.itm_bits = itm_threshold(io.strike, io.call != 0);
    A.min_itm = io.min_itm;
    A.df = reinterpret_cast<const double*>(base + o_tab);
    A.disc = A.df + M;
    A.beta = reinterpret_cast<double*>(base + o_tab) + 2 * (size_t)M;
    A.fit = reinterpret_cast<int*>(base + o_tab + sizeof(double) * 5 * (size_t)M);
    A.screen = reinterpret_cast<const float4*>(base + o_scr);
    A.strike_f = (float)io.strike;
    A.inv_norm_f = (float)A.inv_norm;
    A.acc = reinterpret_cast<Fx128*>(base + o_acc);
    A.status = reinterpret_cast<int*>(base + o_ctl);
    CUDA_TRY(cudaEventRecord(g_dev.ev0, st));
    CUDA_TRY(launch_lsm_apply(A, grid, st));
    CUDA_TRY(cudaEventRecord(g_dev.ev1, st));
    CUDA_TRY(cudaMemcpyAsync(h, base + o_acc, acc_bytes, cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaMemcpyAsync(h + acc_bytes, base + o_ctl, sizeof(int), cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaMemcpyAsync(h + acc_bytes + 2 * sizeof(int), g_dev.paths, sizeof(float), cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaStreamSynchronize(st));
    float ms = 0;
    CUDA_TRY(cudaEventElapsedTime(&ms, g_dev.ev0, g_dev.ev1));
    int status;
    std::memcpy(&status, h + acc_bytes, sizeof(int));
    if ((rc = lsm_status(status))) return rc;
    lsm_results(reinterpret_cast<const Fx128*>(h), grid, io);
    float s0;
    std::memcpy(&s0, h + acc_bytes + 2 * sizeof(int), sizeof(float));
    io.s0 = s0;
    io.paths = N;
    io.grid = grid;
    io.sim_ms = sim_ms;
    io.lsm_ms = ms;
    return THOTH_GPU_OK;
}

// fit up to LSM_MAX_CONTRACTS policies on the stored paths in one launch (lsm_fit_kernel);
// each pass gets its sums and policy, and the launch's device time
int lsm_fit_batch_locked(const Plan& P, double sim_ms, LsmPass* const* io, int C)
{
    int rc = THOTH_GPU_OK;
    if (C < 1 || C > LSM_MAX_CONTRACTS) return fail(THOTH_GPU_E_INVALID, "bad batch of exercise fits");
    int Tmax = 0;
    for (int k = 0; k < C; k++) {
        if ((rc = lsm_check(P, *io[k]))) return rc;
        Tmax = std::max(Tmax, io[k]->M);
    }
    const int64_t N = P.paths;
    const int cap = lsm_fit_max_grid(g_dev.sms);
    if (cap < 1) return fail(THOTH_GPU_E_CUDA, "no resident CTA for the exercise fit kernel");
    const int grid = (int)std::max<int64_t>(1, std::min<int64_t>((N + LSM_THREADS - 1) / LSM_THREADS, cap));
    const int64_t threads = (int64_t)grid * LSM_THREADS;
    const int64_t seg_len = 32 * ((N + threads - 1) / threads);
    const size_t n_list = (size_t)(grid * (LSM_THREADS / 32)) * (size_t)seg_len;
    const size_t acc_bytes = sizeof(Fx128) * (size_t)grid * LSM_NACC;
    // layout: [contracts][tables of every contract] (uploaded) | per contract: cf, val, lists,
    // totals, result rows | control
    size_t o = 0;
    auto take = [&](size_t bytes) {
        const size_t at = o;
        o = align256(o + bytes);
        return at;
    };
    const size_t o_ct = take(sizeof(LsmContract) * C);
    std::vector<size_t> o_tab(C);
    for (int k = 0; k < C; k++) o_tab[k] = take(lsm_tab_bytes(io[k]->M));
    const size_t up_bytes = o;
    const size_t o_zero = o;
    std::vector<size_t> o_tot(C);
    for (int k = 0; k < C; k++) o_tot[k] = take(sizeof(unsigned long long) * 3 * (size_t)io[k]->M * LSM_PART);
    const size_t o_ctl = take(16);
    const size_t zero_bytes = o - o_zero;
    std::vector<size_t> o_cf(C), o_val(C), o_cm(C), o_civ(C), o_cidx(C), o_acc(C);
    for (int k = 0; k < C; k++) {
        o_cf[k] = take(sizeof(double) * (size_t)N);
        o_val[k] = take(sizeof(double) * (size_t)N);
        o_cm[k] = take(sizeof(double) * n_list);
        o_civ[k] = take(sizeof(double) * n_list);
        o_cidx[k] = take(sizeof(int32_t) * n_list);
        o_acc[k] = take(acc_bytes);
    }
    rc = ensure_lsm(o);
    if (rc) return rc;
    size_t back = sizeof(int) + sizeof(float);
    for (int k = 0; k < C; k++) back += acc_bytes + lsm_tab_bytes(io[k]->M);
    rc = ensure_pinned(std::max(up_bytes, back));
    if (rc) return rc;
    unsigned char* base = g_dev.lsm;
    unsigned char* h = g_dev.pinned;
    LsmContract* ct = reinterpret_cast<LsmContract*>(h + o_ct);
    for (int k = 0; k < C; k++) {
        const LsmPass& q = *io[k];
        const int M = q.M;
        lsm_fill_tab(h + o_tab[k], q);
        LsmContract& K = ct[k];
        K.M = M;
        K.call = q.call;
        K.min_itm = q.min_itm;
        K.itm_bits = itm_threshold(q.strike, q.call != 0);
        K.strike = q.strike;
        K.norm = q.norm;
        K.inv_norm = 1.0 / q.norm;
        K.df = reinterpret_cast<const double*>(base + o_tab[k]);
        K.disc = K.df + M;
        K.beta = reinterpret_cast<double*>(base + o_tab[k]) + 2 * (size_t)M;
        K.fit = reinterpret_cast<int*>(base + o_tab[k] + sizeof(double) * 5 * (size_t)M);
        K.cf = reinterpret_cast<double*>(base + o_cf[k]);
        K.val = reinterpret_cast<double*>(base + o_val[k]);
        K.c_idx = reinterpret_cast<int32_t*>(base + o_cidx[k]);
        K.c_m = reinterpret_cast<double*>(base + o_cm[k]);
        K.c_iv = reinterpret_cast<double*>(base + o_civ[k]);
        K.tot = reinterpret_cast<unsigned long long*>(base + o_tot[k]);
        K.acc = reinterpret_cast<Fx128*>(base + o_acc[k]);
    }
    cudaStream_t st = g_dev.stream;
    CUDA_TRY(cudaMemcpyAsync(base, h, up_bytes, cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaMemsetAsync(base + o_zero, 0, zero_bytes, st));
    LsmFitArgs A;
    A.S = g_dev.paths;
    A.ld = P.paths;
    A.n = N;
    A.C = C;
    A.Tmax = Tmax;
    A.ct = reinterpret_cast<const LsmContract*>(base + o_ct);
    A.seg_len = seg_len;
    A.bar = reinterpret_cast<unsigned*>(base + o_ctl);
    A.done = reinterpret_cast<unsigned*>(base + o_ctl + 4);
    A.status = reinterpret_cast<int*>(base + o_ctl + 8);
    CUDA_TRY(cudaEventRecord(g_dev.ev0, st));
    CUDA_TRY(launch_lsm_fit(A, grid, st));
    CUDA_TRY(cudaEventRecord(g_dev.ev1, st));
    size_t hb = 0;
    CUDA_TRY(cudaMemcpyAsync(h + hb, base + o_ctl + 8, sizeof(int), cudaMemcpyDeviceToHost, st));
    hb += sizeof(int);
    CUDA_TRY(cudaMemcpyAsync(h + hb, g_dev.paths, sizeof(float), cudaMemcpyDeviceToHost, st));
    hb += sizeof(float);
    std::vector<size_t> h_acc(C), h_tab(C);
    for (int k = 0; k < C; k++) {
        h_acc[k] = hb;
        CUDA_TRY(cudaMemcpyAsync(h + hb, base + o_acc[k], acc_bytes, cudaMemcpyDeviceToHost, st));
        hb += acc_bytes;
        h_tab[k] = hb;
        CUDA_TRY(cudaMemcpyAsync(h + hb, base + o_tab[k], lsm_tab_bytes(io[k]->M), cudaMemcpyDeviceToHost, st));
        hb += lsm_tab_bytes(io[k]->M);
    }
    CUDA_TRY(cudaStreamSynchronize(st));
    float ms = 0;
    CUDA_TRY(cudaEventElapsedTime(&ms, g_dev.ev0, g_dev.ev1));
    int status;
    std::memcpy(&status, h, sizeof(int));
    if ((rc = lsm_status(status))) return rc;
    float s0;
    std::memcpy(&s0, h + sizeof(int), sizeof(float));
    for (int k = 0; k < C; k++) {
        LsmPass& q = *io[k];
        const int M = q.M;
        // unaligned pinned offsets: copy the sums out before reading them
        std::vector<Fx128> acc((size_t)grid * LSM_NACC);
        std::memcpy(acc.data(), h + h_acc[k], acc_bytes);
        lsm_results(acc.data(), grid, q);
        q.beta.resize(3 * (size_t)M);
        q.fit_at.resize(M);
        std::memcpy(q.beta.data(), h + h_tab[k] + sizeof(double) * 2 * M, sizeof(double) * 3 * M);
        std::memcpy(q.fit_at.data(), h + h_tab[k] + sizeof(double) * 5 * M, sizeof(int32_t) * M);
        q.s0 = s0;
        q.paths = N;
        q.grid = grid;
        q.sim_ms = k == 0 ? sim_ms : 0.0;
        q.lsm_ms = k == 0 ? ms : 0.0; // one launch for the batch: its time on the first pass
    }
    return THOTH_GPU_OK;
}

// simulate the book once with the paths of `asset` stored, then run every pass on them
int lsm_passes_locked(const ThothBookDesc* book, int asset, LsmPass* io, int n)
{
    Plan P;
    double sim_ms = 0;
    int rc = simulate_device_locked(book, asset, P, &sim_ms);
    if (rc) return rc;
    // the fits in batches of LSM_MAX_CONTRACTS launches, the frozen-policy applies one by one
    std::vector<LsmPass*> fits;
    for (int k = 0; k < n; k++) {
        if (io[k].asset != asset) return fail(THOTH_GPU_E_INVALID, "exercise pass on another asset's paths");
        if (io[k].fit) fits.push_back(&io[k]);
    }
    bool first = true;
    for (size_t b = 0; b < fits.size(); b += LSM_MAX_CONTRACTS) {
        const int C = (int)std::min<size_t>(LSM_MAX_CONTRACTS, fits.size() - b);
        rc = lsm_fit_batch_locked(P, first ? sim_ms : 0.0, fits.data() + b, C);
        if (rc) return rc;
        first = false;
    }
    for (int k = 0; k < n; k++) {
        if (io[k].fit) continue;
        rc = lsm_apply_locked(P, first ? sim_ms : 0.0, io[k]);
        if (rc) return rc;
        first = false;
    }
    return THOTH_GPU_OK;
}

} // namespace

// ---------------------------------------------------------------------------
// Allocation-free pricing (thoth_gpu_price_book_noalloc): everything the book
// kernel reads or writes besides the caller's host buffers lives in this one
// statically allocated device array. Host code may not use its name as a
// device address; the address is looked up per device with cudaGetSymbolAddress.
// ---------------------------------------------------------------------------
static __device__ __align__(256) unsigned char g_noalloc_scratch[THOTH_NOALLOC_SCRATCH_BYTES];

static constexpr int kMaxDevices = 64;
static unsigned char* g_noalloc_ptr[kMaxDevices] = {};

// once per device, with that device current. The address is cached for the life of the
// process: a context reset (cudaDeviceReset) between calls is not supported.
static int noalloc_address(int dev, unsigned char** out)
{
    if (dev < 0 || dev >= kMaxDevices) return fail(THOTH_GPU_E_NODEVICE, "device index out of range");
    if (!g_noalloc_ptr[dev]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return fail(THOTH_GPU_E_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
        g_noalloc_ptr[dev] = static_cast<unsigned char*>(p);
    }
    *out = g_noalloc_ptr[dev];
    return THOTH_GPU_OK;
}

static int price_noalloc_locked(const ThothBookDesc* book, ThothBookResult* out)
{
    if (!out) return fail(THOTH_GPU_E_INVALID, "null result");
    int dev = 0, count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) return fail(THOTH_GPU_E_NODEVICE, "no CUDA device");
    // once the engine is bound to a device (any earlier call of the other entry points), this
    // call prices on that device as they do; before that, on the calling thread's current one
    if (g_dev.ready) CUDA_TRY(cudaSetDevice(g_dev.id));
    CUDA_TRY(cudaGetDevice(&dev));
    // a cancel requested before the call ends it here, as at the first tile of the other entry points
    if (g_dev.ready && *(volatile int*)g_dev.cancel_host) return fail(THOTH_GPU_E_CANCELLED, "pricing cancelled");
    cudaDeviceProp prop;
    CUDA_TRY(cudaGetDeviceProperties(&prop, dev));
    if (!(prop.major == 10 && prop.minor == 3))
        return fail(THOTH_GPU_E_NODEVICE, std::string("device ") + prop.name + " is not sm_103 (built for sm_103a only)");
    unsigned char* base = nullptr;
    int rc = noalloc_address(dev, &base);
    if (rc) return rc;
    Plan P;
    rc = build_plan(book, P);
    if (rc) return rc;
    // direction numbers of the book's Sobol dimensions, from the embedded table
    std::vector<uint32_t> V, lo;
    if (!build_direction_numbers(V)) return fail(THOTH_GPU_E_INVALID, "embedded Joe-Kuo table is corrupt");
    const int dims = std::max(P.dp.sobol_dims, 1);
    const size_t v_bytes = sizeof(uint32_t) * 32 * (size_t)dims;
    const size_t lo_bytes = std::max(low_bytes(P), sizeof(uint32_t));
    const size_t n_acc = (size_t)P.dp.n_acc;
    auto up = [](size_t x) { return (x + 255) & ~size_t(255); };
    const size_t o_v = up(P.blob.bytes.size());
    const size_t o_lo = o_v + up(v_bytes);
    const size_t o_out = o_lo + up(lo_bytes);
    const size_t o_st = o_out + up(sizeof(double) * n_acc);
    const size_t o_acc = o_st + 256;
    const size_t row = sizeof(double) * n_acc;
    if (o_acc + row > THOTH_NOALLOC_SCRATCH_BYTES)
        return fail(THOTH_GPU_E_TOO_LARGE, "book needs " + std::to_string(o_acc + row) +
                                               " bytes of device scratch; the allocation-free entry point holds " +
                                               std::to_string((size_t)THOTH_NOALLOC_SCRATCH_BYTES));
    // as many CTA rows of FP64 sums as the array still holds (at most the normal persistent grid)
    const int64_t fit = (int64_t)((THOTH_NOALLOC_SCRATCH_BYTES - o_acc) / row);
    const int64_t full = (int64_t)book_occupancy(P.variant, P.shape, P.smem) * prop.multiProcessorCount;
    const int grid = (int)std::max<int64_t>(1, std::min(std::min(full, fit), P.dp.n_tiles));
    CUDA_TRY(cudaMemcpy(base, P.blob.bytes.data(), P.blob.bytes.size(), cudaMemcpyHostToDevice));
    CUDA_TRY(cudaMemcpy(base + o_v, V.data(), v_bytes, cudaMemcpyHostToDevice));
    {
        // the book's low words in consumption order, built here rather than gathered
        std::vector<uint32_t> all;
        build_low_table(V, dims, all);
        const int* order = reinterpret_cast<const int*>(P.blob.bytes.data() + P.o_sord);
        lo.assign(lo_bytes / sizeof(uint32_t), 0u);
        for (int j = 0; j < P.dp.n_sobol; j++)
            std::memcpy(lo.data() + (size_t)j * P.T, all.data() + (size_t)order[j] * SOBOL_LO_ROW,
                        sizeof(uint32_t) * P.T);
    }
    CUDA_TRY(cudaMemcpy(base + o_lo, lo.data(), lo_bytes, cudaMemcpyHostToDevice));
    CUDA_TRY(cudaMemset(base + o_st, 0, sizeof(int))); // status must start at zero; the sums are zeroed by the kernel
    bind(P, base);
    P.dp.sobol_v = reinterpret_cast<const uint32_t*>(base + o_v);
    bind_low(P, base + o_lo);
    // the engine's host-mapped cancel word, where the engine set it up (it needs no allocation
    // here); the kernel reads it at every tile
    P.dp.cancel = g_dev.ready ? g_dev.cancel_dev : nullptr;
    P.dp.acc = reinterpret_cast<double*>(base + o_acc);
    P.dp.status = reinterpret_cast<int*>(base + o_st);
    CUDA_TRY(launch_book(P.dp, P.variant, P.shape, grid, P.smem, 0));
    CUDA_TRY(launch_reduce(P.dp.acc, grid, (int)n_acc, reinterpret_cast<double*>(base + o_out), 0));
    std::vector<double> o(n_acc);
    int status = 0;
    CUDA_TRY(cudaMemcpy(o.data(), base + o_out, sizeof(double) * n_acc, cudaMemcpyDeviceToHost));
    CUDA_TRY(cudaMemcpy(&status, base + o_st, sizeof(int), cudaMemcpyDeviceToHost));
    if (status != 0) return fail(THOTH_GPU_E_CANCELLED, "pricing cancelled");
    const double n = (double)P.paths;
    const double nan = std::nan("");
    for (int p = 0; p < P.n_products; p++) {
        const double* a = o.data() + 6 * (size_t)p;
        if (out->premium) out->premium[p] = a[0] / n;
        if (out->trust) out->trust[p] = trust_of(a[0], a[1], n);
        const bool dok = (P.greek_mask[p] & 1) != 0, vok = (P.greek_mask[p] & 2) != 0;
        if (out->delta) out->delta[p] = dok ? a[2] / n : nan;
        if (out->delta_trust) out->delta_trust[p] = dok ? trust_of(a[2], a[3], n) : nan;
        if (out->vega) out->vega[p] = vok ? a[4] / n : nan;
        if (out->vega_trust) out->vega_trust[p] = vok ? trust_of(a[4], a[5], n) : nan;
    }
    out->book_premium = o[6 * (size_t)P.n_products] / n;
    out->book_trust = trust_of(o[6 * (size_t)P.n_products], o[6 * (size_t)P.n_products + 1], n);
    out->device_ms = nan;
    out->h2d_bytes = (int64_t)(P.blob.bytes.size() + v_bytes + lo_bytes + sizeof(int));
    out->d2h_bytes = (int64_t)(sizeof(double) * n_acc + sizeof(int));
    return THOTH_GPU_OK;
}

// ---------------------------------------------------------------------------
// Ragged batches: every book's plan in one upload, the whole batch captured once
// into a CUDA graph and replayed while the batch's shapes repeat, all sums back
// in one copy. By default the single-asset books run in one persistent launch
// (batch_kernel): one work list of every book's items (item r of a book = what
// CTA r of the book's own launch does), largest items first, taken by resident
// CTAs from a counter; one gather of the books' low Sobol words before it and
// one fixed-order reduction of all books' rows after it. Books that kernel does
// not run (several assets, or more shared memory than keeps its CTAs resident)
// get their own launches on side streams meanwhile. The other mode launches each
// book's gather, kernel and reduction on one of several streams.
// ---------------------------------------------------------------------------
struct BatchCache {
    int streams_wanted = 8;
    int policy = 0;     // grid policy of every book in the batch (grid_policy)
    int shape = -1;     // per-book mode: launch shape of every single-asset book (-1: each book's own)
    int persistent = 1; // 1: the single-asset books in one persistent launch
    std::vector<cudaStream_t> streams;
    std::vector<cudaEvent_t> events;
    cudaGraphExec_t exec = nullptr;
    std::string signature;
    unsigned char* dev = nullptr;
    size_t dev_size = 0;
    unsigned char* host = nullptr; // pinned
    size_t host_size = 0;
    int replays = 0;
    int launches = 0; // kernel launches recorded into the cached graph
};
static BatchCache g_batch;

static int ensure_batch_streams()
{
    while ((int)g_batch.streams.size() < g_batch.streams_wanted) {
        cudaStream_t s;
        cudaEvent_t e;
        CUDA_TRY(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
        CUDA_TRY(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        g_batch.streams.push_back(s);
        g_batch.events.push_back(e);
    }
    return THOTH_GPU_OK;
}

// the persistent launch of a batch: its books (positions into the plans, decreasing item
// cost), grid and shared memory, and where its tables sit in the batch's device buffer
struct BatchLaunch {
    std::vector<int> books;
    std::vector<char> member; // [n] 1: the book runs in the persistent launch
    int items = 0, grid = 0, max_acc = 0;
    size_t smem = 0;
    size_t o_plans = 0, o_books = 0, o_gather = 0, o_reduce = 0, o_next = 0;
};

static double batch_cost(const Plan& P) { return (double)P.paths * P.dp.n_steps * std::max(1, P.dp.n_assets); }

// the cost of one work item of a book in the persistent launch: its tiles x steps, weighted
// by the model's arithmetic per path-step (GBM one normal, Heston two and the QE step, LSV
// those and the leverage lookup)
static double item_cost(const Plan& P, int grid)
{
    const double w = (P.variant == 0 || P.variant == 5) ? 1.0 : P.variant == 2 ? 4.0 : 3.0;
    const double tiles = (double)((P.dp.n_tiles + grid - 1) / std::max(grid, 1));
    return tiles * P.T * P.dp.n_steps * w;
}

// the batch's device work as recorded into the graph: zero the status words (and the work
// counter), then either the persistent launch with the other books on side streams, or each
// book's gather, kernel and reduction on the stream chosen by a longest-processing-time
// schedule (books by decreasing path-steps, each onto the stream with the least work so far)
static int record_batch(std::vector<Plan>& plans, const std::vector<int>& grid, const std::vector<size_t>& o_out,
                        size_t o_sts, int S, cudaStream_t st, const BatchLaunch* BL)
{
    const int n = (int)plans.size();
    int launches = 0;
    CUDA_TRY(cudaMemsetAsync(g_batch.dev + o_sts, 0, sizeof(int) * (size_t)(n + 1), st));
    std::vector<int> order;
    for (int b = 0; b < n; b++)
        if (!BL || !BL->member[b]) order.push_back(b);
    std::stable_sort(order.begin(), order.end(),
                     [&](int a, int c) { return batch_cost(plans[a]) > batch_cost(plans[c]); });
    if (BL) {
        CUDA_TRY(launch_gather_low_batch(g_dev.sobol_lo, g_batch.dev + BL->o_gather, n, st));
        launches++;
        for (int b = 0; b < n; b++)
            if (plans[b].dp.n_tail > 0) {
                CUDA_TRY(tail_normals(plans[b], st));
                launches++;
            }
    }
    const int side = BL ? (int)std::min<size_t>(order.size(), (size_t)S) : S;
    CUDA_TRY(cudaEventRecord(g_batch.events[0], st));
    for (int k = 0; k < side; k++) CUDA_TRY(cudaStreamWaitEvent(g_batch.streams[k], g_batch.events[0], 0));
    std::vector<double> load(std::max(side, 1), 0.0);
    for (int b : order) {
        const int k = (int)(std::min_element(load.begin(), load.end()) - load.begin());
        load[k] += batch_cost(plans[b]);
        cudaStream_t s = g_batch.streams[k];
        if (!BL) {
            CUDA_TRY(gather_low(plans[b], s));
            launches += plans[b].dp.n_tail > 0 ? 2 : 1;
        }
        CUDA_TRY(launch_book(plans[b].dp, plans[b].variant, plans[b].shape, grid[b], plans[b].smem, s));
        launches++;
        if (!BL) {
            CUDA_TRY(launch_reduce(plans[b].dp.acc, grid[b], plans[b].dp.n_acc,
                                   reinterpret_cast<double*>(g_batch.dev + o_out[b]), s));
            launches++;
        }
    }
    if (BL && !BL->books.empty()) {
        CUDA_TRY(launch_batch_kernel(reinterpret_cast<const DevPlan*>(g_batch.dev + BL->o_plans),
                                     reinterpret_cast<const BatchBook*>(g_batch.dev + BL->o_books),
                                     (int)BL->books.size(), BL->items, reinterpret_cast<int*>(g_batch.dev + BL->o_next),
                                     BL->grid, BL->smem, st));
        launches++;
    }
    for (int k = 0; k < side; k++) {
        CUDA_TRY(cudaEventRecord(g_batch.events[k], g_batch.streams[k]));
        CUDA_TRY(cudaStreamWaitEvent(st, g_batch.events[k], 0));
    }
    if (BL) {
        CUDA_TRY(launch_reduce_batch(g_batch.dev + BL->o_reduce, n, BL->max_acc, st));
        launches++;
    }
    g_batch.launches = launches;
    return THOTH_GPU_OK;
}

static int price_batch_locked(const ThothBookDesc* books, int n, ThothBookResult* out)
{
    int rc = ensure_device();
    if (rc) return rc;
    if (n == 0) return THOTH_GPU_OK;
    rc = ensure_batch_streams();
    if (rc) return rc;
    const bool pers = g_batch.persistent != 0 && n <= 65535; // the batched gather / reduction grids
    const int S = std::min(g_batch.streams_wanted, n);
    std::vector<Plan> plans(n);
    std::vector<int> grid(n);
    std::vector<size_t> o_blob(n), o_lo(n), o_acc(n), o_out(n), o_st(n);
    size_t off = 0;
    auto up = [](size_t x) { return (x + 255) & ~size_t(255); };
    std::string sig = std::to_string(n) + ":" + std::to_string(S) + ":" + std::to_string(g_batch.policy) + ":" +
                      std::to_string(g_batch.shape) + ":" + std::to_string(pers ? 1 : 0);
    // the persistent launch: the books it runs, those whose (8, 2) plan keeps its CTAs resident at
    // their register-bound count; the others keep their own (tuned or default) shape and launch
    const int full = pers ? batch_occupancy(0) : 0;
    std::vector<char> member(n, 0);
    auto joins = [&](const Plan& P) {
        return full > 0 && batch_variant(P.variant) && P.shape == 0 && P.T == batch_tile_paths() &&
               batch_occupancy(P.smem) >= full;
    };
    for (int b = 0; b < n; b++) {
        rc = build_plan(&books[b], plans[b], pers ? -1 : g_batch.shape);
        if (rc) return fail(rc, "book " + std::to_string(b) + ": " + g_err);
        if (pers && batch_variant(plans[b].variant) && plans[b].shape != 0) {
            Plan q;
            rc = build_plan(&books[b], q, 0);
            if (rc) return fail(rc, "book " + std::to_string(b) + ": " + g_err);
            if (joins(q)) plans[b] = std::move(q);
        }
        member[b] = pers && joins(plans[b]);
        grid[b] = grid_for(plans[b], g_batch.policy);
        o_blob[b] = off;
        off += up(plans[b].blob.bytes.size());
        o_lo[b] = off;
        off += up(low_bytes(plans[b]));
        o_acc[b] = off;
        off += up(sizeof(double) * (size_t)grid[b] * plans[b].dp.n_acc);
        sig += "|" + std::to_string(plans[b].variant) + "," + std::to_string(plans[b].shape) + "," +
               std::to_string(grid[b]) + "," +
               std::to_string(plans[b].smem) + "," + std::to_string(plans[b].blob.bytes.size()) + "," +
               std::to_string(plans[b].dp.n_acc) + "," + std::to_string(plans[b].dp.n_tiles);
    }
    // the persistent launch: its books' work-list order, its grid and its tables
    BatchLaunch BL;
    if (pers) {
        BL.member = member;
        for (int b = 0; b < n; b++)
            if (member[b]) {
                BL.books.push_back(b);
                BL.smem = std::max(BL.smem, plans[b].smem);
            }
        std::stable_sort(BL.books.begin(), BL.books.end(), [&](int a, int c) {
            return item_cost(plans[a], grid[a]) > item_cost(plans[c], grid[c]);
        });
        for (int b : BL.books) BL.items += grid[b];
        BL.grid = std::max(1, std::min(full * g_dev.sms, BL.items));
        for (int b = 0; b < n; b++) BL.max_acc = std::max(BL.max_acc, plans[b].dp.n_acc);
        BL.o_plans = off;
        off += up(sizeof(DevPlan) * BL.books.size());
        BL.o_books = off;
        off += up(sizeof(BatchBook) * BL.books.size());
        BL.o_gather = off;
        off += up(sizeof(BatchGather) * (size_t)n);
        BL.o_reduce = off;
        off += up(sizeof(BatchReduce) * (size_t)n);
        sig += "|persistent " + std::to_string(BL.grid) + "," + std::to_string(BL.smem) + "," +
               std::to_string(BL.items);
        for (int b : BL.books) sig += "," + std::to_string(b);
    }
    // outputs and status words (then the work counter) contiguous at the end: one device->host copy
    const size_t o_outs = off;
    size_t cur = o_outs;
    for (int b = 0; b < n; b++) {
        o_out[b] = cur;
        cur += sizeof(double) * plans[b].dp.n_acc;
    }
    cur = up(cur);
    const size_t o_sts = cur;
    for (int b = 0; b < n; b++) o_st[b] = o_sts + sizeof(int) * (size_t)b;
    BL.o_next = o_sts + sizeof(int) * (size_t)n;
    const size_t total = o_sts + up(sizeof(int) * (size_t)(n + 1));
    const size_t back = total - o_outs;
    // device and pinned buffers (a new size invalidates the cached graph)
    if (total > g_batch.dev_size) {
        if (g_batch.exec) cudaGraphExecDestroy(g_batch.exec);
        g_batch.exec = nullptr;
        g_batch.signature.clear();
        if (g_batch.dev) cudaFree(g_batch.dev);
        g_batch.dev = nullptr;
        g_batch.dev_size = 0; // stays empty if the allocation fails
        CUDA_TRY(dev_alloc(&g_batch.dev, total));
        g_batch.dev_size = total;
    }
    if (std::max(o_outs, back) > g_batch.host_size) {
        if (g_batch.host) cudaFreeHost(g_batch.host);
        g_batch.host = nullptr;
        g_batch.host_size = 0;
        CUDA_TRY(host_alloc(&g_batch.host, std::max(o_outs, back)));
        g_batch.host_size = std::max(o_outs, back);
    }
    for (int b = 0; b < n; b++) {
        std::memcpy(g_batch.host + o_blob[b], plans[b].blob.bytes.data(), plans[b].blob.bytes.size());
        bind(plans[b], g_batch.dev + o_blob[b]);
        bind_low(plans[b], g_batch.dev + o_lo[b]);
        plans[b].dp.acc = reinterpret_cast<double*>(g_batch.dev + o_acc[b]);
        plans[b].dp.status = reinterpret_cast<int*>(g_batch.dev + o_st[b]);
        // the kernel parameters are baked into the graph: a replay needs them byte-equal
        sig.append(reinterpret_cast<const char*>(&plans[b].dp), sizeof(DevPlan));
    }
    if (pers) {
        // the persistent launch's tables, uploaded with the plans
        int first = 0;
        for (size_t k = 0; k < BL.books.size(); k++) {
            const int b = BL.books[k];
            std::memcpy(g_batch.host + BL.o_plans + sizeof(DevPlan) * k, &plans[b].dp, sizeof(DevPlan));
            BatchBook bb{(int)k, plans[b].variant, grid[b], first};
            std::memcpy(g_batch.host + BL.o_books + sizeof(BatchBook) * k, &bb, sizeof bb);
            first += grid[b];
        }
        for (int b = 0; b < n; b++) {
            const Plan& P = plans[b];
            BatchGather g{P.dp.sobol_order, const_cast<uint32_t*>(P.dp.sobol_lo), P.dp.n_sobol, P.T};
            std::memcpy(g_batch.host + BL.o_gather + sizeof(BatchGather) * (size_t)b, &g, sizeof g);
            BatchReduce r{P.dp.acc, reinterpret_cast<double*>(g_batch.dev + o_out[b]), grid[b], P.dp.n_acc};
            std::memcpy(g_batch.host + BL.o_reduce + sizeof(BatchReduce) * (size_t)b, &r, sizeof r);
        }
    }
    cudaStream_t st = g_dev.stream;
    CUDA_TRY(cudaMemcpyAsync(g_batch.dev, g_batch.host, o_outs, cudaMemcpyHostToDevice, st));
    if (g_batch.signature != sig || !g_batch.exec) {
        if (g_batch.exec) cudaGraphExecDestroy(g_batch.exec);
        g_batch.exec = nullptr;
        g_batch.signature.clear();
        // kernel attributes are set outside the capture
        for (int b = 0; b < n; b++) occupancy_of(plans[b]);
        CUDA_TRY(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
        rc = record_batch(plans, grid, o_out, o_sts, S, st, pers ? &BL : nullptr);
        cudaGraph_t graph = nullptr;
        const cudaError_t ec = cudaStreamEndCapture(st, &graph); // always leave capture mode
        if (rc) {
            if (graph) cudaGraphDestroy(graph);
            cudaGetLastError();
            return rc;
        }
        if (ec != cudaSuccess) return fail(THOTH_GPU_E_CUDA, std::string("cudaStreamEndCapture: ") + cudaGetErrorString(ec));
        const cudaError_t e = cudaGraphInstantiate(&g_batch.exec, graph, 0);
        cudaGraphDestroy(graph);
        if (e != cudaSuccess) return fail(THOTH_GPU_E_CUDA, std::string("cudaGraphInstantiate: ") + cudaGetErrorString(e));
        g_batch.signature = sig;
        g_batch.replays = 0;
    } else {
        g_batch.replays++;
    }
    CUDA_TRY(cudaEventRecord(g_dev.ev0, st));
    CUDA_TRY(cudaGraphLaunch(g_batch.exec, st));
    CUDA_TRY(cudaEventRecord(g_dev.ev1, st));
    CUDA_TRY(cudaMemcpyAsync(g_batch.host, g_batch.dev + o_outs, back, cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaStreamSynchronize(st));
    float ms = 0;
    CUDA_TRY(cudaEventElapsedTime(&ms, g_dev.ev0, g_dev.ev1));
    const double nan = std::nan("");
    for (int b = 0; b < n; b++) {
        const Plan& P = plans[b];
        int status;
        std::memcpy(&status, g_batch.host + (o_st[b] - o_outs), sizeof(int));
        if (status == 1) return fail(THOTH_GPU_E_CANCELLED, "pricing cancelled");
        const double* o = reinterpret_cast<const double*>(g_batch.host + (o_out[b] - o_outs));
        const double np_ = (double)P.paths;
        ThothBookResult* r = &out[b];
        for (int p = 0; p < P.n_products; p++) {
            const double* a = o + 6 * (size_t)p;
            if (r->premium) r->premium[p] = a[0] / np_;
            if (r->trust) r->trust[p] = trust_of(a[0], a[1], np_);
            const bool dok = (P.greek_mask[p] & 1) != 0, vok = (P.greek_mask[p] & 2) != 0;
            if (r->delta) r->delta[p] = dok ? a[2] / np_ : nan;
            if (r->delta_trust) r->delta_trust[p] = dok ? trust_of(a[2], a[3], np_) : nan;
            if (r->vega) r->vega[p] = vok ? a[4] / np_ : nan;
            if (r->vega_trust) r->vega_trust[p] = vok ? trust_of(a[4], a[5], np_) : nan;
        }
        r->book_premium = o[6 * (size_t)P.n_products] / np_;
        r->book_trust = trust_of(o[6 * (size_t)P.n_products], o[6 * (size_t)P.n_products + 1], np_);
        r->device_ms = ms; // the whole batch's device time
        r->h2d_bytes = b == 0 ? (int64_t)o_outs : 0;
        r->d2h_bytes = b == 0 ? (int64_t)back : 0;
    }
    return THOTH_GPU_OK;
}

// ---------------------------------------------------------------------------
// Autotuner: times candidate launch configurations on the device with CUDA
// events and keeps the fastest. Book level: the persistent grid (k x SMs for
// k = 1 .. resident CTAs per SM, and the balanced grid of each), stored per
// (variant, resident CTAs per SM, tiles). Batch level: the stream count and
// the grid policy of the batch graph.
// ---------------------------------------------------------------------------
static int autotune_book_locked(const ThothBookDesc* book, int reps, ThothTuneResult* out)
{
    int rc = ensure_device();
    if (rc) return rc;
    cudaStream_t st = g_dev.stream;
    double best = 1e300, def_ms = 0;
    int best_g = 1, def_g = 1, count = 0;
    TuneChoice choice;
    TuneKey key;
    Plan best_plan;
    for (int shape = 0;; shape++) {
        Plan P;
        rc = build_plan(book, P, shape);
        if (rc) return rc;
        if (shape >= book_shape_count(P.variant)) break;
        key = tune_key(P.base_variant, P.paths, P.dp.n_steps);
        const int per_sm = occupancy_of(P);
        const int64_t tiles = P.dp.n_tiles;
        // candidates: k x SMs for k = 1 .. resident CTAs per SM, and the balanced grid of each
        std::vector<std::pair<int, int>> cand; // (k, policy)
        std::vector<int> grids;
        for (int k = 1; k <= per_sm; k++)
            for (int pol = 0; pol < 2; pol++) {
                const int g = grid_policy(tiles, (int64_t)k * g_dev.sms, pol);
                if (std::find(grids.begin(), grids.end(), g) == grids.end()) {
                    grids.push_back(g);
                    cand.push_back({k, pol});
                }
            }
        const int gmax = *std::max_element(grids.begin(), grids.end());
        const Layout L = layout_of(P, gmax);
        rc = ensure_arena(L.total);
        if (rc) return rc;
        CUDA_TRY(cudaMemcpy(g_dev.arena, P.blob.bytes.data(), P.blob.bytes.size(), cudaMemcpyHostToDevice));
        bind(P, g_dev.arena);
        bind_low(P, g_dev.arena + L.o_lo);
        CUDA_TRY(gather_low(P, st));
        P.dp.acc = reinterpret_cast<double*>(g_dev.arena + L.o_acc);
        P.dp.status = reinterpret_cast<int*>(g_dev.arena + L.o_st);
        for (size_t c = 0; c < grids.size(); c++) {
            const int g = grids[c];
            CUDA_TRY(cudaMemsetAsync(g_dev.arena + L.o_st, 0, sizeof(int), st));
            CUDA_TRY(launch_book(P.dp, P.variant, P.shape, g, P.smem, st)); // warm-up
            CUDA_TRY(cudaEventRecord(g_dev.ev0, st));
            for (int r = 0; r < reps; r++) {
                CUDA_TRY(launch_book(P.dp, P.variant, P.shape, g, P.smem, st));
                CUDA_TRY(launch_reduce(P.dp.acc, g, P.dp.n_acc, reinterpret_cast<double*>(g_dev.arena + L.o_out), st));
            }
            CUDA_TRY(cudaEventRecord(g_dev.ev1, st));
            CUDA_TRY(cudaStreamSynchronize(st));
            int status = 0;
            CUDA_TRY(cudaMemcpy(&status, g_dev.arena + L.o_st, sizeof(int), cudaMemcpyDeviceToHost));
            if (status == 1) return fail(THOTH_GPU_E_CANCELLED, "autotune cancelled");
            float ms = 0;
            CUDA_TRY(cudaEventElapsedTime(&ms, g_dev.ev0, g_dev.ev1));
            const double per = ms / reps;
            count++;
            if (shape == 0 && g == grid_policy(tiles, (int64_t)per_sm * g_dev.sms, 0)) { // the untuned launch
                def_ms = per;
                def_g = g;
            }
            if (per < best) {
                best = per;
                best_g = g;
                choice.shape = shape;
                choice.per_sm = cand[c].first;
                choice.policy = cand[c].second;
                best_plan.variant = P.variant;
                best_plan.shape = P.shape;
                best_plan.T = P.T;
            }
        }
    }
    g_tuned[key] = choice;
    if (out) {
        out->grid = best_g;
        out->default_grid = def_g;
        out->candidates = count;
        out->streams = 0;
        out->policy = choice.policy;
        out->shape = choice.shape;
        out->threads = book_shape_threads(best_plan.variant, best_plan.shape);
        out->tile_paths = best_plan.T;
        out->best_ms = best;
        out->default_ms = def_ms;
        out->persistent = 0;
    }
    return THOTH_GPU_OK;
}

static int autotune_batch_locked(const ThothBookDesc* books, int n, int reps, ThothTuneResult* out)
{
    std::vector<ThothBookResult> res(std::max(n, 1));
    std::memset(res.data(), 0, sizeof(ThothBookResult) * res.size());
    const int keep_s = g_batch.streams_wanted, keep_p = g_batch.policy, keep_h = g_batch.shape,
              keep_x = g_batch.persistent;
    auto time_one = [&](int X, int S, int pol, int shape, double* ms) {
        g_batch.persistent = X;
        g_batch.streams_wanted = S;
        g_batch.policy = pol;
        g_batch.shape = shape;
        int rc = price_batch_locked(books, n, res.data()); // capture + warm-up
        if (rc) return rc;
        double sum = 0;
        for (int r = 0; r < reps; r++) {
            rc = price_batch_locked(books, n, res.data());
            if (rc) return rc;
            sum += res[0].device_ms;
        }
        *ms = sum / reps;
        return THOTH_GPU_OK;
    };
    double best = 1e300, def_ms = 0;
    int best_s = keep_s, best_p = 0, best_h = -1, best_x = 1, count = 0;
    auto restore = [&](int rc) {
        g_batch.persistent = keep_x;
        g_batch.streams_wanted = keep_s;
        g_batch.policy = keep_p;
        g_batch.shape = keep_h;
        return rc;
    };
    auto consider = [&](double ms, int X, int S, int pol, int shape) {
        count++;
        if (ms < best) {
            best = ms;
            best_x = X;
            best_s = S;
            best_p = pol;
            best_h = shape;
        }
    };
    // 1. the persistent launch (the default) under each grid policy of its books
    for (int pol : {0, 1, 2}) {
        double ms;
        const int rc = time_one(1, keep_s, pol, -1, &ms);
        if (rc) return restore(rc);
        if (pol == 0) def_ms = ms;
        consider(ms, 1, keep_s, pol, -1);
    }
    // 2. one launch per book: stream count, with each book's own shape and the full grid
    int per_s = keep_s;
    double per_best = 1e300;
    for (int S : {1, 2, 4, 8, 16, 32}) {
        if (S > std::max(n, 1) && S != 1) break;
        double ms;
        const int rc = time_one(0, S, 0, -1, &ms);
        if (rc) return restore(rc);
        consider(ms, 0, S, 0, -1);
        if (ms < per_best) {
            per_best = ms;
            per_s = S;
        }
    }
    // 3. one launch shape for every single-asset book, then the grid policy
    int per_h = -1;
    for (int h = 0; h < 4; h++) {
        double ms;
        const int rc = time_one(0, per_s, 0, h, &ms);
        if (rc) return restore(rc);
        consider(ms, 0, per_s, 0, h);
        if (ms < per_best) {
            per_best = ms;
            per_h = h;
        }
    }
    for (int pol : {1, 2}) {
        double ms;
        const int rc = time_one(0, per_s, pol, per_h, &ms);
        if (rc) return restore(rc);
        consider(ms, 0, per_s, pol, per_h);
    }
    g_batch.persistent = best_x;
    g_batch.streams_wanted = best_s;
    g_batch.policy = best_p;
    g_batch.shape = best_h;
    if (out) {
        out->grid = 0;
        out->default_grid = 0;
        out->candidates = count;
        out->streams = best_s;
        out->policy = best_p;
        out->shape = best_h;
        out->threads = 0;
        out->tile_paths = 0;
        out->best_ms = best;
        out->default_ms = def_ms;
        out->persistent = best_x;
    }
    return THOTH_GPU_OK;
}

// autotune cache file: one line per choice, tied to the device it was measured on
static int autotune_save_locked(const char* path)
{
    int rc = ensure_device();
    if (rc) return rc;
    FILE* f = std::fopen(path, "w");
    if (!f) return fail(THOTH_GPU_E_INVALID, std::string("cannot write ") + path);
    std::fprintf(f, "thoth-autotune 1\ndevice %d %s\n", g_dev.sms, g_dev.name.c_str());
    std::fprintf(f, "batch %d %d %d %d\n", g_batch.streams_wanted, g_batch.policy, g_batch.shape,
                 g_batch.persistent);
    for (const auto& kv : g_tuned)
        std::fprintf(f, "book %d %d %d %d %d %d\n", std::get<0>(kv.first), std::get<1>(kv.first), std::get<2>(kv.first),
                     kv.second.shape, kv.second.per_sm, kv.second.policy);
    const bool ok = std::fclose(f) == 0;
    return ok ? THOTH_GPU_OK : fail(THOTH_GPU_E_INVALID, std::string("cannot write ") + path);
}

static int autotune_load_locked(const char* path)
{
    int rc = ensure_device();
    if (rc) return rc;
    FILE* f = std::fopen(path, "r");
    if (!f) return fail(THOTH_GPU_E_INVALID, std::string("cannot read ") + path);
    char line[512];
    int version = 0, sms = -1;
    std::string name;
    std::map<TuneKey, TuneChoice> books;
    int streams = g_batch.streams_wanted, policy = g_batch.policy, bshape = g_batch.shape, pers = g_batch.persistent;
    bool bad = false;
    while (std::fgets(line, sizeof line, f)) {
        int a, b, c, e, g, h;
        char nm[400];
        if (std::sscanf(line, "thoth-autotune %d", &a) == 1) version = a;
        else if (std::sscanf(line, "device %d %399[^\n]", &a, nm) == 2) { sms = a; name = nm; }
        else if (std::sscanf(line, "batch %d %d %d %d", &a, &b, &c, &e) == 4) {
            streams = a;
            policy = b;
            bshape = c;
            pers = e;
        } else if (std::sscanf(line, "batch %d %d %d", &a, &b, &c) == 3) { streams = a; policy = b; bshape = c; }
        else if (std::sscanf(line, "batch %d %d", &a, &b) == 2) { streams = a; policy = b; bshape = -1; }
        else if (std::sscanf(line, "book %d %d %d %d %d %d", &a, &b, &c, &e, &g, &h) == 6) {
            if (a < 0 || a > 6 || e < 0 || e >= book_shape_count(a) || g < 0 || h < 0 || h > 1) bad = true;
            TuneChoice ch;
            ch.shape = e;
            ch.per_sm = g;
            ch.policy = h;
            books[TuneKey(a, b, c)] = ch;
        } else if (line[0] != '\n') bad = true;
    }
    std::fclose(f);
    if (version != 1 || bad || streams < 1 || streams > 64 || policy < 0 || policy > 2 || bshape < -1 ||
        bshape >= book_shape_count(0) || pers < 0 || pers > 1)
        return fail(THOTH_GPU_E_INVALID, std::string("malformed autotune file ") + path);
    if (sms != g_dev.sms || name != g_dev.name)
        return fail(THOTH_GPU_E_UNSUPPORTED, "autotune file was measured on another device (" + name + ")");
    for (const auto& kv : books) g_tuned[kv.first] = kv.second;
    g_batch.streams_wanted = streams;
    g_batch.policy = policy;
    g_batch.shape = bshape;
    g_batch.persistent = pers;
    return THOTH_GPU_OK;
}

struct ThothBookHandle {
    Plan plan;
    int grid = 1;
    Layout layout{};
    unsigned char* dev = nullptr;
};

// LSV leverage calibration (calib.cu): validate, derive the per-date step tables on the
// host (the reference's ACT/365 fractions and exp(-kappa dt) rounded by the host libm),
// upload, one cooperative launch, layers back
int calibrate_locked(ThothLeverageCalib* c)
{
    if (!c) return fail(THOTH_GPU_E_INVALID, "null argument");
    const int n = c->n_dates, pts = c->points;
    const int P = c->particles > 0 ? c->particles : 16384;
    const int bins = c->bins > 0 ? c->bins : 30;
    const int min_count = c->min_bin_count > 0 ? c->min_bin_count : 20;
    if (n < 1 || pts < 2 || !c->days || !c->carry || !c->ln_step || !c->offset || !c->local_vol || !c->leverage)
        return fail(THOTH_GPU_E_INVALID, "calibration needs dates, carries, layer grids, local vols and an output");
    if (c->days[0] != 0) return fail(THOTH_GPU_E_INVALID, "days[0] must be 0 (today)");
    for (int k = 1; k < n; k++)
        if (c->days[k] <= c->days[k - 1]) return fail(THOTH_GPU_E_INVALID, "days must increase");
    if (bins > CALIB_MAX_BINS) return fail(THOTH_GPU_E_INVALID, "at most 128 bins");
    if (P > (1 << 30)) return fail(THOTH_GPU_E_TOO_LARGE, "at most 2^30 particles");
    if (!(c->spot > 0) || !(c->v0 >= 0) || !(c->kappa > 0) || !(c->xi >= 0) || !(c->theta >= 0) ||
        !(c->rho >= -1 && c->rho <= 1))
        return fail(THOTH_GPU_E_INVALID, "bad Heston base or spot");
    for (int k = 0; k < n; k++)
        if (!(c->ln_step[k] > 0)) return fail(THOTH_GPU_E_INVALID, "layer grid spacing must be positive");
    int rc = ensure_device();
    if (rc) return rc;
    std::vector<double> dt(n, 0.0), carry(n, 0.0), qe(n, 1.0);
    for (int k = 1; k < n; k++) {
        dt[k] = (double)(c->days[k] - c->days[k - 1]) / 365.0;
        carry[k] = c->carry[k] * ((double)c->days[k] / 365.0) - c->carry[k - 1] * ((double)c->days[k - 1] / 365.0);
        qe[k] = std::exp(-c->kappa * dt[k]);
    }
    uint64_t jpow[CALIB_JUMP_BITS][4], jdate[4];
    for (int i = 0; i < CALIB_JUMP_BITS; i++)
        if (!xo_jump_poly(1ull << i, jpow[i])) return fail(THOTH_GPU_E_INVALID, "Rng jump polynomial unavailable");
    if (!xo_jump_poly(2ull * (uint64_t)P - 2, jdate)) return fail(THOTH_GPU_E_INVALID, "Rng jump polynomial unavailable");
    std::vector<uint64_t> jtab(CALIB_JTAB_WORDS);
    xo_jump_table(jdate, jtab.data());
    const size_t smem = sizeof(uint64_t) * CALIB_JTAB_WORDS + sizeof(double) * (size_t)pts;
    const int cap = calib_max_grid(g_dev.sms, smem);
    if (cap < 1) return fail(THOTH_GPU_E_TOO_LARGE, "layer too large for shared memory");
    const int grid = std::max(1, std::min(cap, (P + CALIB_THREADS - 1) / CALIB_THREADS));
    // device layout: inputs | layers | ensemble | generators | partial sums | control
    const size_t nd = (size_t)n, np = (size_t)P, npt = (size_t)pts;
    size_t o = 0;
    auto take = [&](size_t bytes) {
        const size_t at = o;
        o = align256(o + bytes);
        return at;
    };
    const size_t o_dt = take(8 * nd), o_carry = take(8 * nd), o_qe = take(8 * nd), o_ls = take(8 * nd);
    const size_t o_off = take(8 * nd), o_lv = take(8 * nd * npt), o_jp = take(8 * 4 * CALIB_JUMP_BITS),
                 o_jt = take(8 * CALIB_JTAB_WORDS);
    const size_t up_bytes = o; // everything above is uploaded in one copy
    const size_t o_lev = take(8 * nd * npt), o_spot = take(8 * np), o_var = take(8 * np), o_lns = take(8 * np);
    const size_t o_rng = take(8 * 4 * np), o_bc = take(8 * 4);
    // per-date totals: zeroed (sums, counts, control) or set to the neutral keys (extremes)
    const size_t o_kmin = take(8 * nd), o_kmax = take(8 * nd);
    const size_t o_zero = o, o_vsum = take(sizeof(Fx128) * nd), o_bcnt = take(4 * nd * (size_t)bins);
    const size_t o_bsum = take(sizeof(Fx128) * nd * (size_t)bins), o_ctl = take(16);
    if (o > g_dev.calib_size) {
        if (g_dev.calib) cudaFree(g_dev.calib);
        g_dev.calib = nullptr;
        g_dev.calib_size = 0;
        CUDA_TRY(dev_alloc(&g_dev.calib, o));
        g_dev.calib_size = o;
    }
    rc = ensure_pinned(std::max(up_bytes, 8 * nd * npt + 16));
    if (rc) return rc;
    unsigned char* h = g_dev.pinned;
    std::memset(h, 0, up_bytes);
    std::memcpy(h + o_dt, dt.data(), 8 * nd);
    std::memcpy(h + o_carry, carry.data(), 8 * nd);
    std::memcpy(h + o_qe, qe.data(), 8 * nd);
    std::memcpy(h + o_ls, c->ln_step, 8 * nd);
    std::memcpy(h + o_off, c->offset, 8 * nd);
    std::memcpy(h + o_lv, c->local_vol, 8 * nd * npt);
    std::memcpy(h + o_jp, jpow, sizeof jpow);
    std::memcpy(h + o_jt, jtab.data(), 8 * CALIB_JTAB_WORDS);
    unsigned char* base = g_dev.calib;
    cudaStream_t st = g_dev.stream;
    CUDA_TRY(cudaMemcpyAsync(base, h, up_bytes, cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaMemsetAsync(base + o_kmin, 0x7f, 8 * nd, st));
    CUDA_TRY(cudaMemsetAsync(base + o_kmax, 0x80, 8 * nd, st));
    CUDA_TRY(cudaMemsetAsync(base + o_zero, 0, o - o_zero, st));
    CalibArgs A;
    A.P = P;
    A.n = n;
    A.points = pts;
    A.bins = bins;
    A.min_count = min_count;
    A.s0 = c->spot;
    A.ln_s0 = std::log(c->spot);
    A.v0 = c->v0;
    A.kappa = c->kappa;
    A.theta = c->theta;
    A.xi = c->xi;
    A.rho = c->rho;
    A.min_cv = c->min_cond_variance > 0 ? c->min_cond_variance : 1e-6;
    A.lmin = c->lev_min > 0 ? c->lev_min : 0.05;
    A.lmax = c->lev_max > 0 ? c->lev_max : 10.0;
    A.dt = reinterpret_cast<const double*>(base + o_dt);
    A.carry = reinterpret_cast<const double*>(base + o_carry);
    A.qe_e = reinterpret_cast<const double*>(base + o_qe);
    A.ln_step = reinterpret_cast<const double*>(base + o_ls);
    A.offset = reinterpret_cast<const int64_t*>(base + o_off);
    A.local_vol = reinterpret_cast<const double*>(base + o_lv);
    A.lev = reinterpret_cast<double*>(base + o_lev);
    A.spot = reinterpret_cast<double*>(base + o_spot);
    A.var = reinterpret_cast<double*>(base + o_var);
    A.lns = reinterpret_cast<double*>(base + o_lns);
    A.rng = reinterpret_cast<uint64_t*>(base + o_rng);
    A.jpow = reinterpret_cast<const uint64_t*>(base + o_jp);
    A.jtab = reinterpret_cast<const uint64_t*>(base + o_jt);
    xo_seed_state(c->seed, A.seed_state);
    A.kmin = reinterpret_cast<long long*>(base + o_kmin);
    A.kmax = reinterpret_cast<long long*>(base + o_kmax);
    A.vsum = reinterpret_cast<Fx128*>(base + o_vsum);
    A.bcnt = reinterpret_cast<unsigned*>(base + o_bcnt);
    A.bsum = reinterpret_cast<Fx128*>(base + o_bsum);
    A.bc = reinterpret_cast<double*>(base + o_bc);
    A.bar = reinterpret_cast<unsigned*>(base + o_ctl);
    A.done = reinterpret_cast<unsigned*>(base + o_ctl + 4);
    A.status = reinterpret_cast<int*>(base + o_ctl + 8);
    A.min_count = min_count;
    CUDA_TRY(cudaEventRecord(g_dev.ev0, st));
    CUDA_TRY(launch_calib(A, grid, smem, st));
    CUDA_TRY(cudaEventRecord(g_dev.ev1, st));
    CUDA_TRY(cudaMemcpyAsync(h, base + o_lev, 8 * nd * npt, cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaMemcpyAsync(h + 8 * nd * npt, base + o_ctl + 8, sizeof(int), cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaStreamSynchronize(st));
    int status;
    std::memcpy(&status, h + 8 * nd * npt, sizeof(int));
    if (status == 2) return fail(THOTH_GPU_E_CUDA, "calibration: a wait timed out");
    if (status == 3) return fail(THOTH_GPU_E_INVALID, "calibration: a variance is out of range (>= 2^36 or negative)");
    if (status != 0) return fail(THOTH_GPU_E_CUDA, "calibration: kernel status " + std::to_string(status));
    std::memcpy(c->leverage, h, 8 * nd * npt);
    float ms = 0;
    CUDA_TRY(cudaEventElapsedTime(&ms, g_dev.ev0, g_dev.ev1));
    c->device_ms = ms;
    return THOTH_GPU_OK;
}

// the exercise passes of thoth_gpu_price_american (american_host.cu)
int thoth_lsm_passes(const ThothBookDesc* book, int asset, LsmPass* io, int n)
{
    try {
        if (!book || (!io && n > 0) || n < 0) return fail(THOTH_GPU_E_INVALID, "null book or passes");
        std::lock_guard<std::mutex> lk(g_mu);
        return lsm_passes_locked(book, asset, io, n);
    } catch (const std::bad_alloc&) {
        return fail(THOTH_GPU_E_NOMEM, "out of host memory");
    } catch (const std::exception& e) {
        return fail(THOTH_GPU_E_INVALID, std::string("host error: ") + e.what());
    }
}

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
extern "C" {

int thoth_gpu_price_book_noalloc(const ThothBookDesc* book, ThothBookResult* out)
{
    try {
        std::lock_guard<std::mutex> lk(g_mu);
        return price_noalloc_locked(book, out);
    } catch (const std::bad_alloc&) {
        return fail(THOTH_GPU_E_NOMEM, "out of host memory");
    } catch (const std::exception& e) {
        return fail(THOTH_GPU_E_INVALID, std::string("host error: ") + e.what());
    }
}

int thoth_gpu_autotune_book(const ThothBookDesc* book, int32_t reps, ThothTuneResult* out)
{
    try {
        if (reps < 1 || reps > 1000) return fail(THOTH_GPU_E_INVALID, "reps must be in [1, 1000]");
        std::lock_guard<std::mutex> lk(g_mu);
        return autotune_book_locked(book, reps, out);
    } catch (const std::bad_alloc&) {
        return fail(THOTH_GPU_E_NOMEM, "out of host memory");
    } catch (const std::exception& e) {
        return fail(THOTH_GPU_E_INVALID, std::string("host error: ") + e.what());
    }
}

int thoth_gpu_autotune_batch(const ThothBookDesc* books, int32_t n_books, int32_t reps, ThothTuneResult* out)
{
    try {
        if (!books || n_books < 1) return fail(THOTH_GPU_E_INVALID, "bad batch");
        if (reps < 1 || reps > 1000) return fail(THOTH_GPU_E_INVALID, "reps must be in [1, 1000]");
        std::lock_guard<std::mutex> lk(g_mu);
        return autotune_batch_locked(books, n_books, reps, out);
    } catch (const std::bad_alloc&) {
        return fail(THOTH_GPU_E_NOMEM, "out of host memory");
    } catch (const std::exception& e) {
        return fail(THOTH_GPU_E_INVALID, std::string("host error: ") + e.what());
    }
}

int thoth_gpu_autotune_save(const char* path)
{
    try {
        if (!path) return fail(THOTH_GPU_E_INVALID, "null path");
        std::lock_guard<std::mutex> lk(g_mu);
        return autotune_save_locked(path);
    } catch (const std::bad_alloc&) {
        return fail(THOTH_GPU_E_NOMEM, "out of host memory");
    } catch (const std::exception& e) {
        return fail(THOTH_GPU_E_INVALID, std::string("host error: ") + e.what());
    }
}

int thoth_gpu_autotune_load(const char* path)
{
    try {
        if (!path) return fail(THOTH_GPU_E_INVALID, "null path");
        std::lock_guard<std::mutex> lk(g_mu);
        return autotune_load_locked(path);
    } catch (const std::bad_alloc&) {
        return fail(THOTH_GPU_E_NOMEM, "out of host memory");
    } catch (const std::exception& e) {
        return fail(THOTH_GPU_E_INVALID, std::string("host error: ") + e.what());
    }
}

int thoth_gpu_autotune_clear(void)
{
    try {
        std::lock_guard<std::mutex> lk(g_mu);
        g_tuned.clear();
        g_batch.streams_wanted = 8;
        g_batch.policy = 0;
        g_batch.shape = -1;
        g_batch.persistent = 1;
        return THOTH_GPU_OK;
    } catch (const std::bad_alloc&) {
        return fail(THOTH_GPU_E_NOMEM, "out of host memory");
    } catch (const std::exception& e) {
        return fail(THOTH_GPU_E_INVALID, std::string("host error: ") + e.what());
    }
}

int thoth_gpu_batch_graph_replays(void)
{
    try {
        std::lock_guard<std::mutex> lk(g_mu);
        return g_batch.replays;
    } catch (const std::bad_alloc&) {
        return fail(THOTH_GPU_E_NOMEM, "out of host memory");
    } catch (const std::exception& e) {
        return fail(THOTH_GPU_E_INVALID, std::string("host error: ") + e.what());
    }
}

int thoth_gpu_book_create(const ThothBookDesc* book, ThothBookHandle** out)
{
    try {
        if (!out) return fail(THOTH_GPU_E_INVALID, "null handle pointer");
        std::lock_guard<std::mutex> lk(g_mu);
        int rc = ensure_device();
        if (rc) return rc;
        ThothBookHandle* h = new ThothBookHandle();
        rc = build_plan(book, h->plan);
        if (rc) {
            delete h;
            return rc;
        }
        h->grid = grid_for(h->plan);
        h->layout = layout_of(h->plan, h->grid);
        cudaError_t e = dev_alloc(&h->dev, h->layout.total);
        if (e != cudaSuccess) {
            delete h;
            return fail(THOTH_GPU_E_NOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
        }
        e = cudaMemcpy(h->dev, h->plan.blob.bytes.data(), h->plan.blob.bytes.size(), cudaMemcpyHostToDevice);
        if (e != cudaSuccess) {
            cudaFree(h->dev);
            delete h;
            return fail(THOTH_GPU_E_CUDA, std::string("cudaMemcpy: ") + cudaGetErrorString(e));
        }
        bind(h->plan, h->dev);
        bind_low(h->plan, h->dev + h->layout.o_lo);
        e = gather_low(h->plan, g_dev.stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(g_dev.stream);
        if (e != cudaSuccess) {
            cudaFree(h->dev);
            delete h;
            return fail(THOTH_GPU_E_CUDA, std::string("gather: ") + cudaGetErrorString(e));
        }
        *out = h;
        return THOTH_GPU_OK;
    } catch (const std::bad_alloc&) {
        return fail(THOTH_GPU_E_NOMEM, "out of host memory");
    } catch (const std::exception& e) {
        return fail(THOTH_GPU_E_INVALID, std::string("host error: ") + e.what());
    }
}

int thoth_gpu_book_run(ThothBookHandle* h, ThothBookResult* out)
{
    try {
        if (!h || !out) return fail(THOTH_GPU_E_INVALID, "null handle or result");
        std::lock_guard<std::mutex> lk(g_mu);
        int rc = ensure_device();
        if (rc) return rc;
        return run_bound(h->plan, h->dev, h->layout, h->grid, out, false);
    } catch (const std::bad_alloc&) {
        return fail(THOTH_GPU_E_NOMEM, "out of host memory");
    } catch (const std::exception& e) {
        return fail(THOTH_GPU_E_INVALID, std::string("host error: ") + e.what());
    }
}

int thoth_gpu_book_destroy(ThothBookHandle* h)
{
    try {
        if (!h) return THOTH_GPU_OK;
        std::lock_guard<std::mutex> lk(g_mu);
        if (h->dev) cudaFree(h->dev);
        delete h;
        return THOTH_GPU_OK;
    } catch (const std::bad_alloc&) {
        return fail(THOTH_GPU_E_NOMEM, "out of host memory");
    } catch (const std::exception& e) {
        return fail(THOTH_GPU_E_INVALID, std::string("host error: ") + e.what());
    }
}

int thoth_gpu_tc_gemm_test(const uint16_t* a, const uint16_t* b, int32_t n, int32_t k, float* d)
{
    try {
        if (!a || !b || !d || n < 16 || n > 256 || n % 16 || k < 16 || k > 256 || k % 16)
            return fail(THOTH_GPU_E_INVALID, "tc gemm test: N, K must be multiples of 16 in [16, 256]");
        std::lock_guard<std::mutex> lk(g_mu);
        int rc = ensure_device();
        if (rc) return rc;
        const size_t ba = (size_t)128 * k * 2, bb = (size_t)n * k * 2, bd = (size_t)128 * n * 4;
        const size_t oa = 0, ob = (ba + 255) & ~size_t(255), od = ob + ((bb + 255) & ~size_t(255)),
                     os = od + ((bd + 255) & ~size_t(255));
        rc = ensure_arena(os + 256);
        if (rc) return rc;
        unsigned char* base = g_dev.arena;
        CUDA_TRY(cudaMemcpyAsync(base + oa, a, ba, cudaMemcpyHostToDevice, g_dev.stream));
        CUDA_TRY(cudaMemcpyAsync(base + ob, b, bb, cudaMemcpyHostToDevice, g_dev.stream));
        CUDA_TRY(cudaMemsetAsync(base + os, 0, sizeof(int), g_dev.stream));
        CUDA_TRY(launch_tc_gemm_test(base + oa, base + ob, n, k, reinterpret_cast<float*>(base + od),
                                     reinterpret_cast<int*>(base + os), g_dev.stream));
        int status = 0;
        CUDA_TRY(cudaMemcpyAsync(d, base + od, bd, cudaMemcpyDeviceToHost, g_dev.stream));
        CUDA_TRY(cudaMemcpyAsync(&status, base + os, sizeof(int), cudaMemcpyDeviceToHost, g_dev.stream));
        CUDA_TRY(cudaStreamSynchronize(g_dev.stream));
        if (status) return fail(THOTH_GPU_E_CUDA, "tensor-core MMA did not complete (bounded wait expired)");
        return THOTH_GPU_OK;
    } catch (const std::bad_alloc&) {
        return fail(THOTH_GPU_E_NOMEM, "out of host memory");
    } catch (const std::exception& e) {
        return fail(THOTH_GPU_E_INVALID, std::string("host error: ") + e.what());
    }
}

int thoth_gpu_measure_fp32_peak(double* tflops, double* ms_out)
{
    try {
        if (!tflops) return fail(THOTH_GPU_E_INVALID, "null output");
        std::lock_guard<std::mutex> lk(g_mu);
        int rc = ensure_device();
        if (rc) return rc;
        rc = ensure_arena(1 << 20);
        if (rc) return rc;
        const int blocks = g_dev.sms * 8, iters = 4096;
        float* d = reinterpret_cast<float*>(g_dev.arena);
        CUDA_TRY(launch_fma_peak(d, blocks, 64, g_dev.stream)); // warm-up
        CUDA_TRY(cudaEventRecord(g_dev.ev0, g_dev.stream));
        CUDA_TRY(launch_fma_peak(d, blocks, iters, g_dev.stream));
        CUDA_TRY(cudaEventRecord(g_dev.ev1, g_dev.stream));
        CUDA_TRY(cudaEventSynchronize(g_dev.ev1));
        float ms = 0;
        CUDA_TRY(cudaEventElapsedTime(&ms, g_dev.ev0, g_dev.ev1));
        const double fmas = (double)blocks * 256 * iters * 16 * 8;
        *tflops = 2.0 * fmas / (ms * 1e-3) / 1e12;
        if (ms_out) *ms_out = ms;
        return THOTH_GPU_OK;
    } catch (const std::bad_alloc&) {
        return fail(THOTH_GPU_E_NOMEM, "out of host memory");
    } catch (const std::exception& e) {
        return fail(THOTH_GPU_E_INVALID, std::string("host error: ") + e.what());
    }
}

int thoth_gpu_measure_mufu_peak(double* gops, double* ms_out)
{
    try {
        if (!gops) return fail(THOTH_GPU_E_INVALID, "null output");
        std::lock_guard<std::mutex> lk(g_mu);
        int rc = ensure_device();
        if (rc) return rc;
        rc = ensure_arena(1 << 20);
        if (rc) return rc;
        const int blocks = g_dev.sms * 8, iters = 1024;
        float* d = reinterpret_cast<float*>(g_dev.arena);
        CUDA_TRY(launch_mufu_peak(d, blocks, 16, g_dev.stream)); // warm-up
        CUDA_TRY(cudaEventRecord(g_dev.ev0, g_dev.stream));
        CUDA_TRY(launch_mufu_peak(d, blocks, iters, g_dev.stream));
        CUDA_TRY(cudaEventRecord(g_dev.ev1, g_dev.stream));
        CUDA_TRY(cudaEventSynchronize(g_dev.ev1));
        float ms = 0;
        CUDA_TRY(cudaEventElapsedTime(&ms, g_dev.ev0, g_dev.ev1));
        const double ops = (double)blocks * 256 * iters * 16 * 8;
        *gops = ops / (ms * 1e-3) / 1e9;
        if (ms_out) *ms_out = ms;
        return THOTH_GPU_OK;
    } catch (const std::bad_alloc&) {
        return fail(THOTH_GPU_E_NOMEM, "out of host memory");
    } catch (const std::exception& e) {
        return fail(THOTH_GPU_E_INVALID, std::string("host error: ") + e.what());
    }
}

int thoth_gpu_debug_fail_allocations(int32_t n)
{
    try {
        if (n < 0) return fail(THOTH_GPU_E_INVALID, "n must be >= 0");
        std::lock_guard<std::mutex> lk(g_mu);
        if (g_dev.ready) {
            // every call has finished its device work before it returned; drop the working
            // buffers so that the next calls allocate them afresh
            CUDA_TRY(cudaSetDevice(g_dev.id));
            CUDA_TRY(cudaDeviceSynchronize());
            if (g_batch.exec) cudaGraphExecDestroy(g_batch.exec);
            g_batch.exec = nullptr;
            g_batch.signature.clear();
            cudaFree(g_batch.dev);
            cudaFreeHost(g_batch.host);
            g_batch.dev = g_batch.host = nullptr;
            g_batch.dev_size = g_batch.host_size = 0;
            cudaFree(g_dev.arena);
            cudaFree(g_dev.paths);
            cudaFree(g_dev.lsm);
            cudaFree(g_dev.calib);
            cudaFreeHost(g_dev.pinned);
            g_dev.arena = g_dev.lsm = g_dev.calib = g_dev.pinned = nullptr;
            g_dev.paths = nullptr;
            g_dev.arena_size = g_dev.paths_size = g_dev.lsm_size = g_dev.calib_size = g_dev.pinned_size = 0;
        }
        g_fail_allocs = n;
        return THOTH_GPU_OK;
    } catch (const std::bad_alloc&) {
        return fail(THOTH_GPU_E_NOMEM, "out of host memory");
    } catch (const std::exception& e) {
        return fail(THOTH_GPU_E_INVALID, std::string("host error: ") + e.what());
    }
}

int thoth_gpu_available(void)
{
    try {
        std::lock_guard<std::mutex> lk(g_mu);
        return ensure_device() == THOTH_GPU_OK ? 1 : 0;
    } catch (const std::bad_alloc&) {
        return fail(THOTH_GPU_E_NOMEM, "out of host memory");
    } catch (const std::exception& e) {
        return fail(THOTH_GPU_E_INVALID, std::string("host error: ") + e.what());
    }
}

int thoth_gpu_device_info(char* buf, size_t n)
{
    try {
        if (!buf || n == 0) return fail(THOTH_GPU_E_INVALID, "null buffer");
        int count = 0;
        std::string s;
        if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) {
            s = "no CUDA device found";
        } else {
            cudaDeviceProp p;
            int dev = 0;
            if (cudaGetDevice(&dev) != cudaSuccess || cudaGetDeviceProperties(&p, dev) != cudaSuccess) {
                s = "CUDA device query failed";
            } else {
                s = std::string(p.name) + " (sm_" + std::to_string(p.major) + std::to_string(p.minor) + ", " +
                    std::to_string(p.multiProcessorCount) + " SMs, " +
                    std::to_string((long long)(p.totalGlobalMem >> 20)) + " MiB)";
            }
        }
        std::snprintf(buf, n, "%s", s.c_str());
        return THOTH_GPU_OK;
    } catch (const std::bad_alloc&) {
        return fail(THOTH_GPU_E_NOMEM, "out of host memory");
    } catch (const std::exception& e) {
        return fail(THOTH_GPU_E_INVALID, std::string("host error: ") + e.what());
    }
}

int thoth_gpu_price_book(const ThothBookDesc* book, ThothBookResult* out)
{
    try {
        std::lock_guard<std::mutex> lk(g_mu);
        return price_locked(book, out);
    } catch (const std::bad_alloc&) {
        return fail(THOTH_GPU_E_NOMEM, "out of host memory");
    } catch (const std::exception& e) {
        return fail(THOTH_GPU_E_INVALID, std::string("host error: ") + e.what());
    }
}

int thoth_gpu_price_european_gbm(double forward, double strike, double t, double vol, double df, int is_call,
                                 int64_t paths, uint64_t seed, ThothGbmResult* out)
{
    try {
        if (!out) return fail(THOTH_GPU_E_INVALID, "null result");
        if (paths <= 0) {
            // reference behaviour for an empty run (mcl_gpu.cu:104-107)
            out->premium = 0.0;
            out->trust = 0.0;
            return THOTH_GPU_OK;
        }
        if (!(t > 0) || !(forward > 0) || !(df > 0) || !(vol >= 0))
            return fail(THOTH_GPU_E_INVALID, "forward, df and t must be > 0 and vol >= 0");
        const double times[2] = {0.0, t};
        const double carry[2] = {0.0, 0.0};
        ThothAsset A;
        std::memset(&A, 0, sizeof A);
        A.model = THOTH_MODEL_GBM;
        A.spot = forward;
        A.carry = carry;
        A.vol = vol;
        ThothProduct Q;
        std::memset(&Q, 0, sizeof Q);
        Q.kind = THOTH_PRODUCT_VANILLA;
        Q.option_type = is_call ? THOTH_CALL : THOTH_PUT;
        Q.asset = 0;
        Q.maturity = 1;
        Q.strike = strike;
        Q.zero_rate = -std::log(df) / t;
        Q.fx = 1.0;
        ThothBookDesc d;
        std::memset(&d, 0, sizeof d);
        d.n_dates = 2;
        d.t = times;
        d.n_assets = 1;
        d.assets = &A;
        d.n_products = 1;
        d.products = &Q;
        d.paths = paths < 2 ? 2 : paths;
        d.use_sobol = (uint64_t)paths < ((uint64_t)1 << 32) ? 1 : 0;
        d.seed = seed;
        double prem = 0, tr = 0;
        ThothBookResult r;
        std::memset(&r, 0, sizeof r);
        r.premium = &prem;
        r.trust = &tr;
        std::lock_guard<std::mutex> lk(g_mu);
        const int rc = price_locked(&d, &r);
        if (rc) return rc;
        out->premium = prem;
        out->trust = tr;
        return THOTH_GPU_OK;
    } catch (const std::bad_alloc&) {
        return fail(THOTH_GPU_E_NOMEM, "out of host memory");
    } catch (const std::exception& e) {
        return fail(THOTH_GPU_E_INVALID, std::string("host error: ") + e.what());
    }
}

int thoth_gpu_sobol_points(int32_t dims, int64_t skip, int64_t n_points, uint32_t* out)
{
    try {
        std::lock_guard<std::mutex> lk(g_mu);
        if (dims < 1 || dims > max_dims() || skip < 0 || n_points < 0 || !out)
            return fail(THOTH_GPU_E_INVALID, "bad Sobol request");
        if ((uint64_t)skip + (uint64_t)n_points >= ((uint64_t)1 << 32)) return fail(THOTH_GPU_E_TOO_LARGE, "index >= 2^32");
        int rc = ensure_device();
        if (rc) return rc;
        const size_t bytes = sizeof(uint32_t) * (size_t)dims * (size_t)n_points;
        rc = ensure_arena(bytes + 256);
        if (rc) return rc;
        uint32_t* d_out = reinterpret_cast<uint32_t*>(g_dev.arena);
        CUDA_TRY(launch_sobol_points(g_dev.sobol_v, dims, skip, n_points, d_out, g_dev.stream));
        CUDA_TRY(cudaMemcpyAsync(out, d_out, bytes, cudaMemcpyDeviceToHost, g_dev.stream));
        CUDA_TRY(cudaStreamSynchronize(g_dev.stream));
        return THOTH_GPU_OK;
    } catch (const std::bad_alloc&) {
        return fail(THOTH_GPU_E_NOMEM, "out of host memory");
    } catch (const std::exception& e) {
        return fail(THOTH_GPU_E_INVALID, std::string("host error: ") + e.what());
    }
}

int thoth_gpu_normal_quantiles(const uint32_t* x, int64_t n, float* out)
{
    try {
        std::lock_guard<std::mutex> lk(g_mu);
        if (n < 0 || (n > 0 && (!x || !out))) return fail(THOTH_GPU_E_INVALID, "bad quantile request");
        int rc = ensure_device();
        if (rc) return rc;
        const size_t bx = ((sizeof(uint32_t) * (size_t)n + 255) & ~size_t(255));
        rc = ensure_arena(bx + sizeof(float) * (size_t)n + 256);
        if (rc) return rc;
        uint32_t* dx = reinterpret_cast<uint32_t*>(g_dev.arena);
        float* dy = reinterpret_cast<float*>(g_dev.arena + bx);
        CUDA_TRY(cudaMemcpyAsync(dx, x, sizeof(uint32_t) * (size_t)n, cudaMemcpyHostToDevice, g_dev.stream));
        CUDA_TRY(launch_quantile(dx, n, dy, g_dev.stream));
        CUDA_TRY(cudaMemcpyAsync(out, dy, sizeof(float) * (size_t)n, cudaMemcpyDeviceToHost, g_dev.stream));
        CUDA_TRY(cudaStreamSynchronize(g_dev.stream));
        return THOTH_GPU_OK;
    } catch (const std::bad_alloc&) {
        return fail(THOTH_GPU_E_NOMEM, "out of host memory");
    } catch (const std::exception& e) {
        return fail(THOTH_GPU_E_INVALID, std::string("host error: ") + e.what());
    }
}

int thoth_gpu_bridge_increments(const double* t, int32_t n_dates, int32_t factors, int64_t skip, int64_t n_paths,
                                float* out)
{
    try {
        std::lock_guard<std::mutex> lk(g_mu);
        if (!t || n_dates < 2 || n_dates > THOTH_MAX_DATES || factors < 1 || factors > 2 || skip < 0 || n_paths < 1 || !out)
            return fail(THOTH_GPU_E_INVALID, "bad bridge request");
        if ((uint64_t)skip + (uint64_t)n_paths >= ((uint64_t)1 << 32)) return fail(THOTH_GPU_E_TOO_LARGE, "index >= 2^32");
        int rc = ensure_device();
        if (rc) return rc;
        std::vector<double> tl(t, t + n_dates);
        for (int i = 1; i < n_dates; i++)
            if (!(tl[i] > tl[i - 1])) return fail(THOTH_GPU_E_INVALID, "t must be strictly increasing");
        BridgeProgram bp;
        std::string err;
        if (!build_bridge(tl, bp, err)) return fail(THOTH_GPU_E_INVALID, err);
        const int N = n_dates - 1;
        std::vector<float> isd(N);
        for (int i = 1; i <= N; i++) isd[i - 1] = (float)(1.0 / std::sqrt(tl[i] - tl[i - 1]));
        Plan P;
        DevPlan& D = P.dp;
        std::memset(&D, 0, sizeof D);
        D.n_steps = N;
        D.n_assets = 1;
        D.ref_factors = factors;
        D.n_factors_active = factors;
        D.stack_factors = factors;
        D.sobol_dims = (int)std::min<long>((long)N * factors, max_dims());
        D.use_sobol = 1;
        D.stack_depth = bp.stack_depth;
        D.skip = skip;
        D.paths = n_paths;
        D.fid_spot[0] = 0;
        D.cidx_spot[0] = 0;
        D.fid_var[0] = factors == 2 ? 1 : -1;
        D.cidx_var[0] = factors == 2 ? 1 : -1;
        const int T = 256;
        D.tile_first = (skip + 1) / T;
        D.n_tiles = (skip + n_paths) / T - (skip + 1) / T + 1;
        P.o_isd = P.blob.put(isd);
        P.o_prog = P.blob.put(bp.prog);
        P.o_nodes = P.blob.put(bp.nodes);
        P.o_recs = P.blob.put(make_recs(bp, isd, std::vector<char>(), factors));
        std::vector<int> order = sobol_order(bp, D);
        D.n_sobol = (int)order.size();
        P.o_sord = P.blob.put(order);
        P.T = T;
        const size_t smem = book_smem_bytes(T, D.sobol_dims, D.stack_depth, factors, 0, 0, 0);
        const size_t o_lo = (P.blob.bytes.size() + 255) & ~size_t(255);
        const size_t o_out = o_lo + ((low_bytes(P) + 255) & ~size_t(255));
        const size_t bytes = sizeof(float) * (size_t)n_paths * factors * N;
        rc = ensure_arena(o_out + bytes + 256);
        if (rc) return rc;
        rc = ensure_pinned(P.blob.bytes.size());
        if (rc) return rc;
        std::memcpy(g_dev.pinned, P.blob.bytes.data(), P.blob.bytes.size());
        CUDA_TRY(cudaMemcpyAsync(g_dev.arena, g_dev.pinned, P.blob.bytes.size(), cudaMemcpyHostToDevice, g_dev.stream));
        D.inv_sqrt_dt = reinterpret_cast<const float*>(g_dev.arena + P.o_isd);
        D.prog = reinterpret_cast<const StepProg*>(g_dev.arena + P.o_prog);
        D.nodes = reinterpret_cast<const BridgeNode*>(g_dev.arena + P.o_nodes);
        D.recs = reinterpret_cast<const StepRec*>(g_dev.arena + P.o_recs);
        D.sobol_v = g_dev.sobol_v;
        D.sobol_order = reinterpret_cast<const int*>(g_dev.arena + P.o_sord);
        bind_low(P, g_dev.arena + o_lo);
        float* d_out = reinterpret_cast<float*>(g_dev.arena + o_out);
        CUDA_TRY(gather_low(P, g_dev.stream));
        const int grid = (int)std::min<int64_t>(D.n_tiles, (int64_t)g_dev.sms * 2);
        CUDA_TRY(launch_bridge(D, grid, smem, d_out, g_dev.stream));
        CUDA_TRY(cudaMemcpyAsync(out, d_out, bytes, cudaMemcpyDeviceToHost, g_dev.stream));
        CUDA_TRY(cudaStreamSynchronize(g_dev.stream));
        return THOTH_GPU_OK;
    } catch (const std::bad_alloc&) {
        return fail(THOTH_GPU_E_NOMEM, "out of host memory");
    } catch (const std::exception& e) {
        return fail(THOTH_GPU_E_INVALID, std::string("host error: ") + e.what());
    }
}

int thoth_gpu_simulate_paths(const ThothBookDesc* book, int32_t asset, float* spots, double* device_ms)
{
    try {
        std::lock_guard<std::mutex> lk(g_mu);
        return simulate_paths_locked(book, asset, spots, device_ms);
    } catch (const std::bad_alloc&) {
        return fail(THOTH_GPU_E_NOMEM, "out of host memory");
    } catch (const std::exception& e) {
        return fail(THOTH_GPU_E_INVALID, std::string("host error: ") + e.what());
    }
}

int thoth_gpu_calibrate_leverage(ThothLeverageCalib* c)
{
    try {
        std::lock_guard<std::mutex> lk(g_mu);
        return calibrate_locked(c);
    } catch (const std::bad_alloc&) {
        return fail(THOTH_GPU_E_NOMEM, "out of host memory");
    } catch (const std::exception& e) {
        return fail(THOTH_GPU_E_INVALID, std::string("host error: ") + e.what());
    }
}

int thoth_gpu_xoshiro_jump(const uint64_t s[4], uint64_t n, uint64_t out[4])
{
    try {
        if (!s || !out) return fail(THOTH_GPU_E_INVALID, "null argument");
        uint64_t poly[4], t[4] = {s[0], s[1], s[2], s[3]};
        if (!xo_jump_poly(n, poly)) return fail(THOTH_GPU_E_INVALID, "jump too long (at most 2^64 - 1 draws)");
        xo_apply_jump(poly, t);
        for (int i = 0; i < 4; i++) out[i] = t[i];
        return THOTH_GPU_OK;
    } catch (const std::exception& e) {
        return fail(THOTH_GPU_E_INVALID, std::string("host error: ") + e.what());
    }
}

int thoth_gpu_price_batch(const ThothBookDesc* books, int32_t n_books, ThothBookResult* out)
{
    try {
        if (!books || !out || n_books < 0) return fail(THOTH_GPU_E_INVALID, "bad batch");
        std::lock_guard<std::mutex> lk(g_mu);
        return price_batch_locked(books, n_books, out);
    } catch (const std::bad_alloc&) {
        return fail(THOTH_GPU_E_NOMEM, "out of host memory");
    } catch (const std::exception& e) {
        return fail(THOTH_GPU_E_INVALID, std::string("host error: ") + e.what());
    }
}

int thoth_gpu_batch_persistent(int32_t on)
{
    try {
        if (on < 0 || on > 1) return fail(THOTH_GPU_E_INVALID, "persistent must be 0 or 1");
        std::lock_guard<std::mutex> lk(g_mu);
        g_batch.persistent = on;
        return THOTH_GPU_OK;
    } catch (const std::bad_alloc&) {
        return fail(THOTH_GPU_E_NOMEM, "out of host memory");
    } catch (const std::exception& e) {
        return fail(THOTH_GPU_E_INVALID, std::string("host error: ") + e.what());
    }
}

int thoth_gpu_batch_launches(void)
{
    try {
        std::lock_guard<std::mutex> lk(g_mu);
        return g_batch.exec ? g_batch.launches : 0;
    } catch (const std::bad_alloc&) {
        return fail(THOTH_GPU_E_NOMEM, "out of host memory");
    } catch (const std::exception& e) {
        return fail(THOTH_GPU_E_INVALID, std::string("host error: ") + e.what());
    }
}

int thoth_gpu_batch_streams(int32_t n)
{
    try {
        if (n < 1 || n > 64) return fail(THOTH_GPU_E_INVALID, "streams must be in [1, 64]");
        std::lock_guard<std::mutex> lk(g_mu);
        g_batch.streams_wanted = n;
        return THOTH_GPU_OK;
    } catch (const std::bad_alloc&) {
        return fail(THOTH_GPU_E_NOMEM, "out of host memory");
    } catch (const std::exception& e) {
        return fail(THOTH_GPU_E_INVALID, std::string("host error: ") + e.what());
    }
}

// no lock: called from another thread while a pricing call holds the mutex
int thoth_gpu_request_cancel(void)
{
    try {
        if (!g_dev.ready) return fail(THOTH_GPU_E_NODEVICE, "engine not initialised");
        *(volatile int*)g_dev.cancel_host = 1;
        return THOTH_GPU_OK;
    } catch (const std::bad_alloc&) {
        return fail(THOTH_GPU_E_NOMEM, "out of host memory");
    } catch (const std::exception& e) {
        return fail(THOTH_GPU_E_INVALID, std::string("host error: ") + e.what());
    }
}

int thoth_gpu_clear_cancel(void)
{
    try {
        if (g_dev.ready) *(volatile int*)g_dev.cancel_host = 0;
        return THOTH_GPU_OK;
    } catch (const std::bad_alloc&) {
        return fail(THOTH_GPU_E_NOMEM, "out of host memory");
    } catch (const std::exception& e) {
        return fail(THOTH_GPU_E_INVALID, std::string("host error: ") + e.what());
    }
}

const char* thoth_gpu_last_error(void) { return g_err.c_str(); }

int thoth_gpu_bridge_program(const double* t, int32_t n_dates, int32_t* first_count, double* nodes, int32_t* n_nodes,
                             int32_t* stack_depth)
{
    try {
        if (!t || n_dates < 2 || n_dates > THOTH_MAX_DATES || !first_count || !nodes || !n_nodes || !stack_depth)
            return fail(THOTH_GPU_E_INVALID, "bad bridge program request");
        std::vector<double> tl(t, t + n_dates);
        for (int i = 1; i < n_dates; i++)
            if (!(tl[i] > tl[i - 1])) return fail(THOTH_GPU_E_INVALID, "t must be strictly increasing");
        BridgeProgram bp;
        std::string err;
        if (!build_bridge(tl, bp, err)) return fail(THOTH_GPU_E_INVALID, err);
        for (size_t i = 0; i < bp.prog.size(); i++) {
            first_count[2 * i] = bp.prog[i].first;
            first_count[2 * i + 1] = bp.prog[i].count;
        }
        for (size_t k = 0; k < bp.nodes.size(); k++) {
            nodes[4 * k] = bp.nodes[k].lw;
            nodes[4 * k + 1] = bp.nodes[k].rw;
            nodes[4 * k + 2] = bp.nodes[k].sd;
            nodes[4 * k + 3] = bp.nodes[k].bstep;
        }
        *n_nodes = (int32_t)bp.nodes.size();
        *stack_depth = bp.stack_depth;
        return THOTH_GPU_OK;
    } catch (const std::bad_alloc&) {
        return fail(THOTH_GPU_E_NOMEM, "out of host memory");
    } catch (const std::exception& e) {
        return fail(THOTH_GPU_E_INVALID, std::string("host error: ") + e.what());
    }
}

int thoth_gpu_plan_summary(const ThothBookDesc* book, int64_t* out)
{
    try {
        if (!out) return fail(THOTH_GPU_E_INVALID, "null output");
        std::lock_guard<std::mutex> lk(g_mu);
        Plan P;
        const int rc = build_plan(book, P);
        if (rc) return rc;
        out[0] = P.variant;
        out[1] = P.T;
        out[2] = (int64_t)P.smem;
        out[3] = P.dp.n_slots_used;
        out[4] = P.dp.n_groups;
        out[5] = P.dp.stack_depth;
        out[6] = P.dp.sobol_dims;
        out[7] = P.dp.n_tiles;
        out[8] = P.shape;
        out[9] = book_shape_threads(P.variant, P.shape);
        out[10] = P.dp.few_m;
        return THOTH_GPU_OK;
    } catch (const std::bad_alloc&) {
        return fail(THOTH_GPU_E_NOMEM, "out of host memory");
    } catch (const std::exception& e) {
        return fail(THOTH_GPU_E_INVALID, std::string("host error: ") + e.what());
    }
}

} // extern "C"
