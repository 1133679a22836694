// surrogate_host.cu — C ABI of the learned Heston surrogate: a 7 -> 4 x 128
// SiLU -> 1 MLP trained and served by the tcgen05 kernels of surrogate.cu.
// No reference counterpart: the reference has no learned pricer.
#include "thoth_gpu.h"

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <new>
#include <stdexcept>
#include <random>
#include <string>
#include <vector>

namespace thoth {
namespace mlp {
struct TrainArgs {
    int rows;
    const __nv_bfloat16* x;
    const float* y;
    const float* inv_w2;
    const float* params;
    const __nv_bfloat16* wbf;
    float* z[5];
    __nv_bfloat16* a[5];
    __nv_bfloat16* dz[5];
    float* part;
    float* loss_part;
    int* status;
};
struct TrainSched {
    long long count, total, steps_per_epoch, step0;
    double lr0;
    float lr_t, bc1, bc2;
    int rows;
    long long decay_steps;
    double lr_lo;
};
} // namespace mlp
cudaError_t mlp_train_step(const mlp::TrainArgs& A, float* params, float* m, float* v, __nv_bfloat16* wbf, float lr,
                           float b1, float b2, float eps, float bc1, float bc2, float* loss_out, cudaStream_t st,
                           const mlp::TrainSched* sched = nullptr);
cudaError_t mlp_train_prepare();
void mlp_sched_init(mlp::TrainSched& s);
cudaError_t mlp_sched_advance(mlp::TrainSched* s, cudaStream_t st);
cudaError_t mlp_weight_avg(const float* params, float* avg, int k, cudaStream_t st);
cudaError_t mlp_mean_add(float* sum, const float* y, int64_t n, int j, int k, cudaStream_t st);
cudaError_t mlp_weight_avg_finish(float* params, const float* avg, __nv_bfloat16* wbf, cudaStream_t st);
cudaError_t mlp_infer(const __nv_bfloat16* x, int n, const float* params, const __nv_bfloat16* wbf, float* y,
                      int* status, int grid, cudaStream_t st);
cudaError_t mlp_gather_batch(const __nv_bfloat16* X, const float* Y, const float* W, const int* perm, int64_t first,
                             int rows, __nv_bfloat16* xb, float* yb, float* wb, cudaStream_t st,
                             const mlp::TrainSched* sched = nullptr);
int mlp_n_params();
int mlp_n_bf();
struct LatticeArgs {
    const double* params;
    const double* lms;
    const double* Ts;
    double lo[7], hi[7];
    double floor;
    int64_t n;
    int n_lm, n_T;
};
cudaError_t lattice_features(const LatticeArgs& A, __nv_bfloat16* x, cudaStream_t st);
cudaError_t lattice_scale(const LatticeArgs& A, const float* y, float* price, cudaStream_t st);
} // namespace thoth

using namespace thoth;

namespace {
thread_local std::string s_err;
std::mutex s_mu;
int sfail(int code, const std::string& m)
{
    s_err = m;
    return code;
}
#define STRY(expr)                                                                                              \
    do {                                                                                                        \
        cudaError_t e_ = (expr);                                                                                \
        if (e_ != cudaSuccess)                                                                                  \
            return sfail(e_ == cudaErrorMemoryAllocation ? THOTH_GPU_E_NOMEM : THOTH_GPU_E_CUDA,                \
                         std::string(#expr) + ": " + cudaGetErrorString(e_));                                    \
    } while (0)

constexpr int H = 128, KIN = 16, NF = 7;
constexpr int OFF_W1 = 0, OFF_B1 = H * KIN, OFF_W2 = OFF_B1 + H, LAYER = H * H + H, OFF_W5 = OFF_W2 + 3 * LAYER,
              OFF_B5 = OFF_W5 + H;

__nv_bfloat16 to_bf(float f)
{
    return __float2bfloat16(f);
}
} // namespace

struct ThothSurrogate {
    int np = 0, nbf = 0;
    float* params = nullptr; // FP32 master
    float* m = nullptr;
    float* v = nullptr;
    __nv_bfloat16* wbf = nullptr;
    int* status = nullptr;
    cudaStream_t st = nullptr;
    int dev = 0; // the device current when the handle was created; every call sets it
    int sms = 0;
    int64_t step = 0;
    // training buffers (grown on demand)
    int cap_rows = 0;
    unsigned char* tb = nullptr;
    mlp::TrainArgs A{};
    float* loss = nullptr;
    // inference buffers
    int64_t cap_inf = 0;
    unsigned char* ib = nullptr;
    // lattice serving: parameter sets and lattice axes, scaled prices
    int64_t cap_lat = 0;
    unsigned char* lb = nullptr;
    // the training schedule the captured step reads (learning rate, bias corrections, batch)
    mlp::TrainSched* sched = nullptr;
    // the running average of the weights over a training call's last epochs
    float* avg = nullptr;
    // device copy of a training set and its per-epoch permutation (grown on demand)
    int64_t cap_ds = 0;
    unsigned char* ds = nullptr;
    int* perm_host = nullptr; // pinned
    cudaEvent_t perm_copied = nullptr;
};

namespace {

void host_params_to_bf(const std::vector<float>& p, std::vector<__nv_bfloat16>& w)
{
    w.assign((size_t)H * KIN + 3 * (size_t)H * H, to_bf(0.f));
    for (int j = 0; j < H * KIN; j++) w[j] = to_bf(p[OFF_W1 + j]);
    for (int l = 0; l < 3; l++)
        for (int j = 0; j < H * H; j++) w[(size_t)H * KIN + (size_t)l * H * H + j] = to_bf(p[OFF_W2 + l * LAYER + j]);
}

int upload_params(ThothSurrogate* s, const std::vector<float>& p)
{
    std::vector<__nv_bfloat16> w;
    host_params_to_bf(p, w);
    STRY(cudaMemcpyAsync(s->params, p.data(), sizeof(float) * s->np, cudaMemcpyHostToDevice, s->st));
    STRY(cudaMemcpyAsync(s->wbf, w.data(), sizeof(__nv_bfloat16) * w.size(), cudaMemcpyHostToDevice, s->st));
    STRY(cudaStreamSynchronize(s->st));
    return THOTH_GPU_OK;
}

int ensure_train(ThothSurrogate* s, int rows)
{
    if (rows <= s->cap_rows) return THOTH_GPU_OK;
    if (s->tb) cudaFree(s->tb);
    s->tb = nullptr;
    s->cap_rows = 0; // stays empty if the allocation fails
    const int tiles = rows / 128;
    size_t off = 0;
    auto take = [&](size_t bytes) {
        const size_t o = off;
        off += (bytes + 255) & ~size_t(255);
        return o;
    };
    const size_t ox = take((size_t)rows * KIN * 2), oy = take((size_t)rows * 4), ow = take((size_t)rows * 4);
    size_t oz[5], oa[5], od[5];
    for (int l = 1; l <= 4; l++) {
        oz[l] = take((size_t)rows * H * 4);
        oa[l] = take((size_t)rows * H * 2);
        od[l] = take((size_t)rows * H * 2);
    }
    const size_t op = take((size_t)tiles * s->np * 4), ol = take((size_t)tiles * 4), oloss = take(4);
    STRY(cudaMalloc(&s->tb, off));
    s->cap_rows = rows;
    mlp::TrainArgs& A = s->A;
    A.x = reinterpret_cast<const __nv_bfloat16*>(s->tb + ox);
    A.y = reinterpret_cast<const float*>(s->tb + oy);
    A.inv_w2 = reinterpret_cast<const float*>(s->tb + ow);
    for (int l = 1; l <= 4; l++) {
        A.z[l] = reinterpret_cast<float*>(s->tb + oz[l]);
        A.a[l] = reinterpret_cast<__nv_bfloat16*>(s->tb + oa[l]);
        A.dz[l] = reinterpret_cast<__nv_bfloat16*>(s->tb + od[l]);
    }
    A.z[0] = nullptr;
    A.a[0] = nullptr;
    A.dz[0] = nullptr;
    A.part = reinterpret_cast<float*>(s->tb + op);
    A.loss_part = reinterpret_cast<float*>(s->tb + ol);
    s->loss = reinterpret_cast<float*>(s->tb + oloss);
    A.params = s->params;
    A.wbf = s->wbf;
    A.status = s->status;
    return THOTH_GPU_OK;
}

// pack rows [i0, i0 + rows) of a (possibly permuted) host dataset into pinned-free host staging
void pack(const float* x, const float* y, const float* scale, const int64_t* idx, int64_t i0, int rows,
          std::vector<__nv_bfloat16>& hx, std::vector<float>& hy, std::vector<float>& hw)
{
    hx.assign((size_t)rows * KIN, to_bf(0.f));
    hy.resize(rows);
    hw.resize(rows);
    for (int r = 0; r < rows; r++) {
        const int64_t i = idx ? idx[i0 + r] : i0 + r;
        for (int f = 0; f < NF; f++) {
            // each feature enters as a bf16 pair hi + lo (columns f and f + 7, tied weights),
            // keeping about 16 significant bits of the input
            const float v = x[i * NF + f];
            const __nv_bfloat16 hi = to_bf(v);
            hx[(size_t)r * KIN + f] = hi;
            hx[(size_t)r * KIN + NF + f] = to_bf(v - __bfloat162float(hi));
        }
        hy[r] = y[i];
        const double sc = scale ? scale[i] : 1.0;
        hw[r] = (float)(1.0 / (sc * sc));
    }
}

int upload_batch(ThothSurrogate* s, const std::vector<__nv_bfloat16>& hx, const std::vector<float>& hy,
                 const std::vector<float>& hw)
{
    mlp::TrainArgs& A = s->A;
    STRY(cudaMemcpyAsync(const_cast<__nv_bfloat16*>(A.x), hx.data(), hx.size() * 2, cudaMemcpyHostToDevice, s->st));
    STRY(cudaMemcpyAsync(const_cast<float*>(A.y), hy.data(), hy.size() * 4, cudaMemcpyHostToDevice, s->st));
    STRY(cudaMemcpyAsync(const_cast<float*>(A.inv_w2), hw.data(), hw.size() * 4, cudaMemcpyHostToDevice, s->st));
    A.a[0] = const_cast<__nv_bfloat16*>(A.x);
    return THOTH_GPU_OK;
}

int check_status(ThothSurrogate* s)
{
    int st = 0;
    STRY(cudaMemcpyAsync(&st, s->status, sizeof(int), cudaMemcpyDeviceToHost, s->st));
    STRY(cudaStreamSynchronize(s->st));
    if (st) return sfail(THOTH_GPU_E_CUDA, "tensor-core MMA did not complete (bounded wait expired)");
    return THOTH_GPU_OK;
}


// one network's training call in three phases, so that several networks can train side by side
struct TrainRun {
    ThothSurrogate* s = nullptr;
    int64_t n = 0, steps_per_epoch = 0, total = 0;
    int epochs = 0, avg_epochs = 0;
    int* dP = nullptr;              // the device permutation of the current epoch
    std::vector<int> idx;           // the host permutation
    std::mt19937_64 rng;
    cudaGraphExec_t exec = nullptr; // one captured step: gather, forward, backward, Adam, loss, schedule
    TrainRun() = default;
    TrainRun(const TrainRun&) = delete;
    TrainRun& operator=(const TrainRun&) = delete;
    ~TrainRun()
    {
        if (exec) cudaGraphExecDestroy(exec);
    }
};

// the training set up once on the member's device memory (bf16 hi/lo inputs, targets, loss
// weights), the schedule of this call, and the captured step
int train_setup(TrainRun& R, ThothSurrogate* s, const float* x, const float* y, const float* scale, int64_t n,
                int epochs, int batch, double lr, uint64_t seed, int avg_epochs, double lr_avg)
{
    R.s = s;
    R.n = n;
    R.epochs = epochs;
    R.avg_epochs = avg_epochs;
    const int B = (int)std::min<int64_t>(batch, n / 128 * 128);
    int rc = ensure_train(s, B);
    if (rc) return rc;
    if (avg_epochs > 0 && !s->avg) STRY(cudaMalloc(&s->avg, sizeof(float) * s->np));
    // each epoch uploads one permutation and every step gathers its rows on the device
    if (n > s->cap_ds) {
        if (s->ds) cudaFree(s->ds);
        if (s->perm_host) cudaFreeHost(s->perm_host);
        s->ds = nullptr;
        s->perm_host = nullptr;
        s->cap_ds = 0;
        STRY(cudaMalloc(&s->ds, (size_t)n * (KIN * 2 + 4 + 4 + 4) + 1024));
        STRY(cudaHostAlloc(&s->perm_host, sizeof(int) * (size_t)n, cudaHostAllocDefault));
        if (!s->perm_copied) STRY(cudaEventCreateWithFlags(&s->perm_copied, cudaEventDisableTiming));
        s->cap_ds = n;
    }
    auto up = [](size_t v) { return (v + 255) & ~size_t(255); };
    __nv_bfloat16* dX = reinterpret_cast<__nv_bfloat16*>(s->ds);
    float* dY = reinterpret_cast<float*>(s->ds + up((size_t)n * KIN * 2));
    float* dW = reinterpret_cast<float*>(reinterpret_cast<unsigned char*>(dY) + up((size_t)n * 4));
    R.dP = reinterpret_cast<int*>(reinterpret_cast<unsigned char*>(dW) + up((size_t)n * 4));
    {
        std::vector<__nv_bfloat16> hx;
        std::vector<float> hy, hw;
        pack(x, y, scale, nullptr, 0, (int)n, hx, hy, hw);
        STRY(cudaMemcpy(dX, hx.data(), hx.size() * 2, cudaMemcpyHostToDevice));
        STRY(cudaMemcpy(dY, hy.data(), hy.size() * 4, cudaMemcpyHostToDevice));
        STRY(cudaMemcpy(dW, hw.data(), hw.size() * 4, cudaMemcpyHostToDevice));
    }
    R.idx.resize(n);
    for (int64_t i = 0; i < n; i++) R.idx[i] = (int)i;
    R.rng.seed(seed);
    R.steps_per_epoch = n / B;
    R.total = R.steps_per_epoch * epochs;
    mlp::TrainArgs& A = s->A;
    A.a[0] = const_cast<__nv_bfloat16*>(A.x);
    A.rows = B;
    // the schedule of this call on the device: the captured step reads its batch offset,
    // learning rate and bias corrections there and advances it
    if (!s->sched) STRY(cudaMalloc(&s->sched, sizeof(mlp::TrainSched)));
    mlp::TrainSched sc{};
    sc.count = 0;
    sc.total = R.total;
    sc.steps_per_epoch = R.steps_per_epoch;
    sc.step0 = s->step;
    sc.lr0 = lr;
    sc.rows = B;
    // without averaging the decay runs over every step down to zero; with it, over the steps
    // before the averaged epochs, down to lr_avg, which then holds
    sc.decay_steps = avg_epochs > 0 ? R.steps_per_epoch * (int64_t)(epochs - avg_epochs) : R.total;
    sc.lr_lo = avg_epochs > 0 ? lr_avg : 0.0;
    if (sc.decay_steps < 1) sc.decay_steps = 1;
    mlp_sched_init(sc);
    STRY(cudaMemcpyAsync(s->sched, &sc, sizeof sc, cudaMemcpyHostToDevice, s->st));
    STRY(cudaMemsetAsync(s->status, 0, sizeof(int), s->st));
    STRY(mlp_train_prepare());
    // one step (gather, forward, backward, Adam, loss, schedule) captured once, replayed
    // for every step: its launches' arguments do not change from step to step
    cudaGraph_t graph = nullptr;
    STRY(cudaStreamBeginCapture(s->st, cudaStreamCaptureModeThreadLocal));
    cudaError_t ce = mlp_gather_batch(dX, dY, dW, R.dP, 0, B, const_cast<__nv_bfloat16*>(A.x),
                                      const_cast<float*>(A.y), const_cast<float*>(A.inv_w2), s->st, s->sched);
    if (ce == cudaSuccess)
        ce = mlp_train_step(A, s->params, s->m, s->v, s->wbf, 0.f, 0.9f, 0.999f, 1e-8f, 1.f, 1.f, s->loss, s->st,
                            s->sched);
    if (ce == cudaSuccess) ce = mlp_sched_advance(s->sched, s->st);
    const cudaError_t ee = cudaStreamEndCapture(s->st, &graph);
    if (ce == cudaSuccess) ce = ee;
    if (ce == cudaSuccess) ce = cudaGraphInstantiate(&R.exec, graph, 0);
    if (graph) cudaGraphDestroy(graph);
    if (ce != cudaSuccess) return sfail(THOTH_GPU_E_CUDA, std::string("training step graph: ") + cudaGetErrorString(ce));
    STRY(cudaEventRecord(s->perm_copied, s->st));
    return THOTH_GPU_OK;
}

// epoch e: the next permutation is drawn on the host while the device runs the previous
// epoch; at the averaged epochs the weights at the epoch's end join the running average
int train_epoch(TrainRun& R, int e)
{
    ThothSurrogate* s = R.s;
    std::shuffle(R.idx.begin(), R.idx.end(), R.rng);
    STRY(cudaEventSynchronize(s->perm_copied)); // the previous permutation has left the pinned buffer
    std::memcpy(s->perm_host, R.idx.data(), sizeof(int) * (size_t)R.n);
    STRY(cudaMemcpyAsync(R.dP, s->perm_host, sizeof(int) * (size_t)R.n, cudaMemcpyHostToDevice, s->st));
    STRY(cudaEventRecord(s->perm_copied, s->st));
    for (int64_t b = 0; b < R.steps_per_epoch; b++) STRY(cudaGraphLaunch(R.exec, s->st));
    if (R.avg_epochs > 0 && e >= R.epochs - R.avg_epochs)
        STRY(mlp_weight_avg(s->params, s->avg, e - (R.epochs - R.avg_epochs), s->st));
    return THOTH_GPU_OK;
}

int train_finish(TrainRun& R, double* final_loss)
{
    ThothSurrogate* s = R.s;
    if (R.avg_epochs > 0) STRY(mlp_weight_avg_finish(s->params, s->avg, s->wbf, s->st));
    s->step += R.total;
    float l = 0;
    STRY(cudaMemcpyAsync(&l, s->loss, sizeof(float), cudaMemcpyDeviceToHost, s->st));
    STRY(cudaStreamSynchronize(s->st));
    const int rc = check_status(s);
    if (rc) return rc;
    if (final_loss) *final_loss = l / s->A.rows;
    return THOTH_GPU_OK;
}

} // namespace

extern "C" {

int thoth_gpu_surrogate_create(ThothSurrogate** out, uint64_t seed)
{
    try {
        if (!out) return sfail(THOTH_GPU_E_INVALID, "null handle pointer");
        std::lock_guard<std::mutex> lk(s_mu);
        int n = 0;
        if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) return sfail(THOTH_GPU_E_NODEVICE, "no CUDA device");
        int dev = 0;
        STRY(cudaGetDevice(&dev));
        cudaDeviceProp p;
        STRY(cudaGetDeviceProperties(&p, dev));
        if (!(p.major == 10 && p.minor == 3)) return sfail(THOTH_GPU_E_NODEVICE, "not an sm_103 device");
        ThothSurrogate* s = new ThothSurrogate();
        s->dev = dev;
        s->np = mlp_n_params();
        s->nbf = mlp_n_bf();
        s->sms = p.multiProcessorCount;
        cudaError_t e = cudaStreamCreateWithFlags(&s->st, cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaMalloc(&s->params, sizeof(float) * s->np * 3);
        if (e == cudaSuccess) e = cudaMalloc(&s->wbf, sizeof(__nv_bfloat16) * s->nbf);
        if (e == cudaSuccess) e = cudaMalloc(&s->status, sizeof(int));
        if (e != cudaSuccess) {
            delete s;
            return sfail(THOTH_GPU_E_NOMEM, std::string("surrogate allocation: ") + cudaGetErrorString(e));
        }
        s->m = s->params + s->np;
        s->v = s->params + 2 * s->np;
        // Xavier-uniform weights, zero biases; W1 only on the 7 real input columns
        std::mt19937_64 rng(seed);
        std::vector<float> h(s->np, 0.f);
        auto fill = [&](int off, int rows, int cols, int fan_in, int used_cols) {
            const double a = std::sqrt(6.0 / (fan_in + rows));
            std::uniform_real_distribution<double> U(-a, a);
            for (int r = 0; r < rows; r++)
                for (int c = 0; c < cols; c++) h[off + r * cols + c] = c < used_cols ? (float)U(rng) : 0.f;
        };
        fill(OFF_W1, H, KIN, NF, NF);
        for (int r = 0; r < H; r++) // tie the lo-part columns to the hi-part columns
            for (int f = 0; f < NF; f++) h[OFF_W1 + r * KIN + NF + f] = h[OFF_W1 + r * KIN + f];
        for (int l = 0; l < 3; l++) fill(OFF_W2 + l * LAYER, H, H, H, H);
        fill(OFF_W5, 1, H, H, H);
        int rc = upload_params(s, h);
        if (rc == THOTH_GPU_OK) {
            e = cudaMemsetAsync(s->m, 0, sizeof(float) * 2 * s->np, s->st);
            if (e == cudaSuccess) e = cudaMemsetAsync(s->status, 0, sizeof(int), s->st);
            if (e == cudaSuccess) e = cudaStreamSynchronize(s->st);
            if (e != cudaSuccess) rc = sfail(THOTH_GPU_E_CUDA, cudaGetErrorString(e));
        }
        if (rc) {
            delete s;
            return rc;
        }
        *out = s;
        return THOTH_GPU_OK;
    } catch (const std::bad_alloc&) {
        return sfail(THOTH_GPU_E_NOMEM, "out of host memory");
    } catch (const std::exception& e) {
        return sfail(THOTH_GPU_E_INVALID, std::string("host error: ") + e.what());
    }
}

int thoth_gpu_surrogate_destroy(ThothSurrogate* s)
{
    try {
        if (!s) return THOTH_GPU_OK;
        std::lock_guard<std::mutex> lk(s_mu);
        cudaSetDevice(s->dev); // frees below whatever this returns
        cudaFree(s->params);
        cudaFree(s->wbf);
        cudaFree(s->status);
        if (s->tb) cudaFree(s->tb);
        if (s->ib) cudaFree(s->ib);
        if (s->lb) cudaFree(s->lb);
        if (s->sched) cudaFree(s->sched);
        if (s->avg) cudaFree(s->avg);
        if (s->ds) cudaFree(s->ds);
        if (s->perm_host) cudaFreeHost(s->perm_host);
        if (s->perm_copied) cudaEventDestroy(s->perm_copied);
        if (s->st) cudaStreamDestroy(s->st);
        delete s;
        return THOTH_GPU_OK;
    } catch (const std::bad_alloc&) {
        return sfail(THOTH_GPU_E_NOMEM, "out of host memory");
    } catch (const std::exception& e) {
        return sfail(THOTH_GPU_E_INVALID, std::string("host error: ") + e.what());
    }
}

int thoth_gpu_surrogate_n_params(void) { return mlp_n_params(); }

int thoth_gpu_surrogate_get_params(ThothSurrogate* s, float* params)
{
    try {
        if (!s || !params) return sfail(THOTH_GPU_E_INVALID, "null argument");
        std::lock_guard<std::mutex> lk(s_mu);
        STRY(cudaSetDevice(s->dev));
        STRY(cudaMemcpyAsync(params, s->params, sizeof(float) * s->np, cudaMemcpyDeviceToHost, s->st));
        STRY(cudaStreamSynchronize(s->st));
        return THOTH_GPU_OK;
    } catch (const std::bad_alloc&) {
        return sfail(THOTH_GPU_E_NOMEM, "out of host memory");
    } catch (const std::exception& e) {
        return sfail(THOTH_GPU_E_INVALID, std::string("host error: ") + e.what());
    }
}

int thoth_gpu_surrogate_set_params(ThothSurrogate* s, const float* params)
{
    try {
        if (!s || !params) return sfail(THOTH_GPU_E_INVALID, "null argument");
        std::lock_guard<std::mutex> lk(s_mu);
        STRY(cudaSetDevice(s->dev));
        std::vector<float> h(params, params + s->np);
        return upload_params(s, h);
    } catch (const std::bad_alloc&) {
        return sfail(THOTH_GPU_E_NOMEM, "out of host memory");
    } catch (const std::exception& e) {
        return sfail(THOTH_GPU_E_INVALID, std::string("host error: ") + e.what());
    }
}

int thoth_gpu_surrogate_gradient(ThothSurrogate* s, const float* x, const float* y, const float* scale, int32_t rows,
                                 float* grad, double* loss)
{
    try {
        if (!s || !x || !y || !grad || rows < 128 || rows % 128) return sfail(THOTH_GPU_E_INVALID, "rows must be a multiple of 128");
        std::lock_guard<std::mutex> lk(s_mu);
        STRY(cudaSetDevice(s->dev));
        int rc = ensure_train(s, rows);
        if (rc) return rc;
        std::vector<__nv_bfloat16> hx;
        std::vector<float> hy, hw;
        pack(x, y, scale, nullptr, 0, rows, hx, hy, hw);
        rc = upload_batch(s, hx, hy, hw);
        if (rc) return rc;
        s->A.rows = rows;
        // a step with lr = 0 leaves the parameters unchanged but fills the partial gradients
        std::vector<float> keep_m(2 * (size_t)s->np);
        STRY(cudaMemcpyAsync(keep_m.data(), s->m, sizeof(float) * 2 * s->np, cudaMemcpyDeviceToHost, s->st));
        STRY(cudaMemsetAsync(s->status, 0, sizeof(int), s->st));
        STRY(mlp_train_step(s->A, s->params, s->m, s->v, s->wbf, 0.f, 0.9f, 0.999f, 1e-8f, 1.f, 1.f, s->loss, s->st));
        rc = check_status(s);
        if (rc) return rc;
        const int tiles = rows / 128;
        std::vector<float> part((size_t)tiles * s->np);
        STRY(cudaMemcpyAsync(part.data(), s->A.part, sizeof(float) * part.size(), cudaMemcpyDeviceToHost, s->st));
        float l = 0;
        STRY(cudaMemcpyAsync(&l, s->loss, sizeof(float), cudaMemcpyDeviceToHost, s->st));
        STRY(cudaMemcpyAsync(s->m, keep_m.data(), sizeof(float) * 2 * s->np, cudaMemcpyHostToDevice, s->st));
        STRY(cudaStreamSynchronize(s->st));
        for (int j = 0; j < s->np; j++) {
            double g = 0;
            for (int t = 0; t < tiles; t++) g += part[(size_t)t * s->np + j];
            grad[j] = (float)g;
        }
        if (loss) *loss = l / rows;
        return THOTH_GPU_OK;
    } catch (const std::bad_alloc&) {
        return sfail(THOTH_GPU_E_NOMEM, "out of host memory");
    } catch (const std::exception& e) {
        return sfail(THOTH_GPU_E_INVALID, std::string("host error: ") + e.what());
    }
}

int thoth_gpu_surrogate_train(ThothSurrogate* s, const float* x, const float* y, const float* scale, int64_t n,
                              int32_t epochs, int32_t batch, double lr, uint64_t seed, double* final_loss)
{
    return thoth_gpu_surrogate_train_avg(s, x, y, scale, n, epochs, batch, lr, seed, 0, 0.0, final_loss);
}

int thoth_gpu_surrogate_train_avg(ThothSurrogate* s, const float* x, const float* y, const float* scale, int64_t n,
                                  int32_t epochs, int32_t batch, double lr, uint64_t seed, int32_t avg_epochs,
                                  double lr_avg, double* final_loss)
{
    return thoth_gpu_surrogate_train_members(&s, 1, x, y, scale, n, epochs, batch, lr, seed, avg_epochs, lr_avg,
                                             final_loss);
}

int thoth_gpu_surrogate_train_members(ThothSurrogate* const* members, int32_t k, const float* x, const float* y,
                                      const float* scale, int64_t n, int32_t epochs, int32_t batch, double lr,
                                      uint64_t seed, int32_t avg_epochs, double lr_avg, double* final_loss)
{
    try {
        if (!members || k < 1 || k > 64 || !x || !y || n < 128 || epochs < 1 || batch < 128 || batch % 128 ||
            !(lr > 0))
            return sfail(THOTH_GPU_E_INVALID, "bad training arguments (batch must be a multiple of 128)");
        if (avg_epochs < 0 || avg_epochs >= epochs || (avg_epochs > 0 && !(lr_avg > 0 && lr_avg <= lr)))
            return sfail(THOTH_GPU_E_INVALID, "bad weight averaging (0 <= avg_epochs < epochs, 0 < lr_avg <= lr)");
        if (n > ((int64_t)1 << 31) - 1) return sfail(THOTH_GPU_E_TOO_LARGE, "training set beyond 2^31 rows");
        for (int j = 0; j < k; j++) {
            if (!members[j]) return sfail(THOTH_GPU_E_INVALID, "null member");
            for (int i = 0; i < j; i++)
                if (members[i] == members[j]) return sfail(THOTH_GPU_E_INVALID, "a member appears twice");
            if (members[j]->dev != members[0]->dev) return sfail(THOTH_GPU_E_INVALID, "members on different devices");
        }
        std::lock_guard<std::mutex> lk(s_mu);
        STRY(cudaSetDevice(members[0]->dev));
        std::vector<TrainRun> runs(k);
        for (int j = 0; j < k; j++) {
            const int rc = train_setup(runs[j], members[j], x, y, scale, n, epochs, batch, lr, seed + (uint64_t)j,
                                       avg_epochs, lr_avg);
            if (rc) return rc;
        }
        // the members' epochs interleaved: each member replays its own step graph on its own stream,
        // so their kernels run side by side on the device
        for (int e = 0; e < epochs; e++)
            for (int j = 0; j < k; j++) {
                const int rc = train_epoch(runs[j], e);
                if (rc) return rc;
            }
        for (int j = 0; j < k; j++) {
            const int rc = train_finish(runs[j], final_loss ? final_loss + j : nullptr);
            if (rc) return rc;
        }
        return THOTH_GPU_OK;
    } catch (const std::bad_alloc&) {
        return sfail(THOTH_GPU_E_NOMEM, "out of host memory");
    } catch (const std::exception& e) {
        return sfail(THOTH_GPU_E_INVALID, std::string("host error: ") + e.what());
    }
}

int thoth_gpu_surrogate_predict(ThothSurrogate* s, const float* x, int64_t n, float* y, double* device_ms)
{
    try {
        if (!s || !x || !y || n < 1 || n > ((int64_t)1 << 30)) return sfail(THOTH_GPU_E_INVALID, "bad predict arguments");
        std::lock_guard<std::mutex> lk(s_mu);
        STRY(cudaSetDevice(s->dev));
        if (n > s->cap_inf) {
            if (s->ib) cudaFree(s->ib);
            s->ib = nullptr;
            s->cap_inf = 0;
            const int64_t cap = (n + 127) / 128 * 128;
            STRY(cudaMalloc(&s->ib, (size_t)cap * (KIN * 2 + 8) + 512));
            s->cap_inf = cap;
        }
        __nv_bfloat16* dx = reinterpret_cast<__nv_bfloat16*>(s->ib);
        float* dy = reinterpret_cast<float*>(s->ib + (size_t)s->cap_inf * KIN * 2);
        std::vector<__nv_bfloat16> hx((size_t)n * KIN, to_bf(0.f));
        for (int64_t i = 0; i < n; i++)
            for (int f = 0; f < NF; f++) {
                const float v = x[i * NF + f];
                const __nv_bfloat16 hi = to_bf(v);
                hx[(size_t)i * KIN + f] = hi;
                hx[(size_t)i * KIN + NF + f] = to_bf(v - __bfloat162float(hi));
            }
        STRY(cudaMemcpyAsync(dx, hx.data(), hx.size() * 2, cudaMemcpyHostToDevice, s->st));
        STRY(cudaMemsetAsync(s->status, 0, sizeof(int), s->st));
        cudaEvent_t e0, e1;
        STRY(cudaEventCreate(&e0));
        STRY(cudaEventCreate(&e1));
        const int tiles = (int)((n + 127) / 128);
        const int grid = std::min(tiles, s->sms);
        STRY(cudaEventRecord(e0, s->st));
        STRY(mlp_infer(dx, (int)n, s->params, s->wbf, dy, s->status, grid, s->st));
        STRY(cudaEventRecord(e1, s->st));
        STRY(cudaMemcpyAsync(y, dy, sizeof(float) * n, cudaMemcpyDeviceToHost, s->st));
        STRY(cudaStreamSynchronize(s->st));
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        if (device_ms) *device_ms = ms;
        return check_status(s);
    } catch (const std::bad_alloc&) {
        return sfail(THOTH_GPU_E_NOMEM, "out of host memory");
    } catch (const std::exception& e) {
        return sfail(THOTH_GPU_E_INVALID, std::string("host error: ") + e.what());
    }
}

int thoth_gpu_surrogate_price_lattice(ThothSurrogate* s, const double* params, int32_t n_sets, const double* lms,
                                      int32_t n_lm, const double* Ts, int32_t n_T, const double* box_lo,
                                      const double* box_hi, double floor, float* prices, double* device_ms)
{
    return thoth_gpu_surrogate_price_lattice_mean(&s, 1, params, n_sets, lms, n_lm, Ts, n_T, box_lo, box_hi, floor,
                                                  prices, device_ms);
}

int thoth_gpu_surrogate_price_lattice_mean(ThothSurrogate* const* members, int32_t k, const double* params,
                                           int32_t n_sets, const double* lms, int32_t n_lm, const double* Ts,
                                           int32_t n_T, const double* box_lo, const double* box_hi, double floor,
                                           float* prices, double* device_ms)
{
    try {
        if (!members || k < 1 || k > 64 || !params || !lms || !Ts || !box_lo || !box_hi || !prices || n_sets < 1 ||
            n_lm < 1 || n_T < 1 || !(floor > 0))
            return sfail(THOTH_GPU_E_INVALID, "bad lattice arguments");
        for (int j = 0; j < k; j++) {
            if (!members[j]) return sfail(THOTH_GPU_E_INVALID, "null member");
            if (members[j]->dev != members[0]->dev) return sfail(THOTH_GPU_E_INVALID, "members on different devices");
        }
        ThothSurrogate* s = members[0]; // its buffers and stream serve the call
        const int64_t n = (int64_t)n_sets * n_lm * n_T;
        if (n > ((int64_t)1 << 30)) return sfail(THOTH_GPU_E_TOO_LARGE, "more than 2^30 lattice cells");
        for (int q = 0; q < 7; q++)
            if (!(box_hi[q] > box_lo[q])) return sfail(THOTH_GPU_E_INVALID, "empty training box");
        std::lock_guard<std::mutex> lk(s_mu);
        STRY(cudaSetDevice(s->dev));
        auto up = [](size_t x) { return (x + 255) & ~size_t(255); };
        if (n > s->cap_inf) {
            if (s->ib) cudaFree(s->ib);
            s->ib = nullptr;
            s->cap_inf = 0;
            const int64_t cap = (n + 127) / 128 * 128;
            STRY(cudaMalloc(&s->ib, (size_t)cap * (KIN * 2 + 8) + 512));
            s->cap_inf = cap;
        }
        const size_t in_bytes = up(sizeof(double) * ((size_t)n_sets * 5 + n_lm + n_T));
        const int64_t need = (int64_t)(in_bytes + up(sizeof(float) * (size_t)n));
        if (need > s->cap_lat) {
            if (s->lb) cudaFree(s->lb);
            s->lb = nullptr;
            s->cap_lat = 0;
            STRY(cudaMalloc(&s->lb, (size_t)need));
            s->cap_lat = need;
        }
        double* dp = reinterpret_cast<double*>(s->lb);
        double* dlm = dp + (size_t)n_sets * 5;
        double* dT = dlm + n_lm;
        float* dprice = reinterpret_cast<float*>(s->lb + in_bytes);
        STRY(cudaMemcpyAsync(dp, params, sizeof(double) * (size_t)n_sets * 5, cudaMemcpyHostToDevice, s->st));
        STRY(cudaMemcpyAsync(dlm, lms, sizeof(double) * n_lm, cudaMemcpyHostToDevice, s->st));
        STRY(cudaMemcpyAsync(dT, Ts, sizeof(double) * n_T, cudaMemcpyHostToDevice, s->st));
        LatticeArgs A{};
        A.params = dp;
        A.lms = dlm;
        A.Ts = dT;
        for (int q = 0; q < 7; q++) {
            A.lo[q] = box_lo[q];
            A.hi[q] = box_hi[q];
        }
        A.floor = floor;
        A.n = n;
        A.n_lm = n_lm;
        A.n_T = n_T;
        __nv_bfloat16* dx = reinterpret_cast<__nv_bfloat16*>(s->ib);
        float* dy = reinterpret_cast<float*>(s->ib + (size_t)s->cap_inf * KIN * 2);
        STRY(cudaMemsetAsync(s->status, 0, sizeof(int), s->st));
        cudaEvent_t e0, e1;
        STRY(cudaEventCreate(&e0));
        STRY(cudaEventCreate(&e1));
        const int tiles = (int)((n + 127) / 128);
        const int grid = std::min(tiles, s->sms);
        STRY(cudaEventRecord(e0, s->st));
        STRY(lattice_features(A, dx, s->st));
        if (k == 1) {
            STRY(mlp_infer(dx, (int)n, s->params, s->wbf, dy, s->status, grid, s->st));
            STRY(lattice_scale(A, dy, dprice, s->st));
        } else {
            // each member's normalised prices, added in member order into the mean
            float* dsum = reinterpret_cast<float*>(s->ib + ((size_t)s->cap_inf * (KIN * 2 + 4) + 255) / 256 * 256);
            for (int j = 0; j < k; j++) {
                STRY(mlp_infer(dx, (int)n, members[j]->params, members[j]->wbf, dy, s->status, grid, s->st));
                STRY(mlp_mean_add(dsum, dy, n, j, k, s->st));
            }
            STRY(lattice_scale(A, dsum, dprice, s->st));
        }
        STRY(cudaEventRecord(e1, s->st));
        STRY(cudaMemcpyAsync(prices, dprice, sizeof(float) * n, cudaMemcpyDeviceToHost, s->st));
        STRY(cudaStreamSynchronize(s->st));
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        if (device_ms) *device_ms = ms;
        return check_status(s);
    } catch (const std::bad_alloc&) {
        return sfail(THOTH_GPU_E_NOMEM, "out of host memory");
    } catch (const std::exception& e) {
        return sfail(THOTH_GPU_E_INVALID, std::string("host error: ") + e.what());
    }
}

const char* thoth_gpu_surrogate_last_error(void) { return s_err.c_str(); }

} // extern "C"
