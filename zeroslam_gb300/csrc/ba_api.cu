// C ABI of the sm_103a bundle adjuster (include/zeroslam_ba.h): the handle,
// the once-per-problem structure analysis and the Levenberg-Marquardt driver
// whose state lives on the device (one small read-back per attempt).
//
// The LM control flow restates factor_graph::solve, source/factor_graph.hpp:489-615
// (gpdaniels/zeroslam): initial damping (:511-522), up to max_failures attempts
// per outer iteration (:541), Cholesky failure -> more damping (:542-551),
// acceptance by the gain ratio (:556-591), rollback of rejected steps
// (:601-605) and the stop rules (:608-611).
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <new>
#include <set>
#include <string>
#include <thread>
#include <condition_variable>
#include <functional>
#include <tuple>
#include <vector>

#include "../../include/zeroslam_ba.h"
#include "ba_internal.h"

using namespace zs;

namespace {

constexpr int kSegment = 512;  // triples per Schur segment (a warp's share)


struct CudaError {
    cudaError_t err;
};

#define ZS_CUDA(x)                                  \
    do {                                            \
        cudaError_t e_ = (x);                       \
        if (e_ != cudaSuccess) throw CudaError{e_}; \
    } while (0)

// Device memory of one problem, allocated in a fixed order. A new problem
// of the same kind reuses the previous problem's buffer at the same position
// when it is large enough (setting a problem of the same shape again, as a
// tracking loop does every frame, then allocates nothing).
struct DevPool {
    std::vector<std::pair<void*, size_t>> slots;  // this problem's buffers, in allocation order
    std::vector<std::pair<void*, size_t>> spare;  // the previous problem's, reusable by position

    void* get(size_t bytes) {
        if (bytes == 0) bytes = 16;
        const size_t i = slots.size();
        if (i < spare.size() && spare[i].first) {
            if (spare[i].second >= bytes) {
                slots.push_back(spare[i]);
                spare[i].first = nullptr;
                return slots.back().first;
            }
            cudaFree(spare[i].first);
            spare[i].first = nullptr;
        }
        void* p = nullptr;
        ZS_CUDA(cudaMalloc(&p, bytes));
        slots.push_back({p, bytes});
        return p;
    }
    // The problem is released; its buffers stay for the next one.
    void recycle() {
        trim();
        spare = std::move(slots);
        slots.clear();
    }
    // Frees the spare buffers no allocation reused.
    void trim() {
        for (auto& e : spare)
            if (e.first) cudaFree(e.first);
        spare.clear();
    }
    void release_all() {
        trim();
        for (auto& e : slots) cudaFree(e.first);
        slots.clear();
    }
};

template <typename T>
T* dalloc(size_t count, DevPool& pool) {
    return static_cast<T*>(pool.get(count * sizeof(T)));
}

template <typename T>
T* upload(const std::vector<T>& v, DevPool& pool, cudaStream_t s) {
    T* d = dalloc<T>(v.size(), pool);
    if (!v.empty()) ZS_CUDA(cudaMemcpyAsync(d, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, s));
    return d;
}

// Host threads for the structure analysis.
int host_threads() {
    static const int n = std::max(1, std::min(16, (int)std::thread::hardware_concurrency()));
    return n;
}

// Persistent workers for the structure analysis (host_threads() - 1 of them,
// shared by all handles; one dispatch at a time, the caller takes part):
// starting threads for each of the analysis's parallel steps cost ~0.3 ms
// per step.
class HostPool {
  public:
    static HostPool& get() {
        static HostPool pool;
        return pool;
    }
    int workers() const { return (int)threads_.size(); }
    // f(t) for t in [0, n), n <= workers() + 1; t = 0 on the calling thread
    void run(int n, const std::function<void(int)>& f) {
        std::lock_guard<std::mutex> one(run_mu_);
        {
            std::lock_guard<std::mutex> lk(mu_);
            task_ = &f;
            ntask_ = n;
            pending_ = (int)threads_.size();
            ++generation_;
        }
        cv_.notify_all();
        f(0);
        std::unique_lock<std::mutex> lk(mu_);
        done_.wait(lk, [&] { return pending_ == 0; });
        task_ = nullptr;
    }
    ~HostPool() {
        {
            std::lock_guard<std::mutex> lk(mu_);
            stop_ = true;
        }
        cv_.notify_all();
        for (auto& t : threads_) t.join();
    }

  private:
    HostPool() {
        for (int i = 1; i < host_threads(); ++i) threads_.emplace_back([this, i] { loop(i); });
    }
    void loop(int id) {
        long long seen = 0;
        for (;;) {
            const std::function<void(int)>* f = nullptr;
            int n = 0;
            {
                std::unique_lock<std::mutex> lk(mu_);
                cv_.wait(lk, [&] { return stop_ || generation_ != seen; });
                if (stop_) return;
                seen = generation_;
                f = task_;
                n = ntask_;
            }
            if (id < n) (*f)(id);
            std::lock_guard<std::mutex> lk(mu_);
            if (--pending_ == 0) done_.notify_one();
        }
    }
    std::vector<std::thread> threads_;
    std::mutex run_mu_, mu_;
    std::condition_variable cv_, done_;
    const std::function<void(int)>* task_ = nullptr;
    int ntask_ = 0, pending_ = 0;
    long long generation_ = 0;
    bool stop_ = false;
};

// f(t, begin, end) on nt threads over [cuts[t], cuts[t + 1]).
template <typename F>
void parallel_ranges(const std::vector<int64_t>& cuts, F f) {
    const int nt = (int)cuts.size() - 1;
    if (nt <= 1) {
        if (nt == 1) f(0, cuts[0], cuts[1]);
        return;
    }
    HostPool& pool = HostPool::get();
    if (nt > pool.workers() + 1) {  // more ranges than threads: each thread takes every k-th
        const int w = pool.workers() + 1;
        pool.run(w, [&](int t) {
            for (int r = t; r < nt; r += w) f(r, cuts[r], cuts[r + 1]);
        });
        return;
    }
    pool.run(nt, [&](int t) { f(t, cuts[t], cuts[t + 1]); });
}

// Cuts [0, n) into nt ranges of about equal weight (prefix[i] = weight of [0, i)).
std::vector<int64_t> balanced_cuts(const std::vector<int64_t>& prefix, int nt) {
    const int64_t n = (int64_t)prefix.size() - 1;
    std::vector<int64_t> cuts{0};
    const int64_t total = prefix[n];
    for (int t = 1; t < nt; ++t) {
        const int64_t target = total * t / nt;
        const int64_t c = std::lower_bound(prefix.begin(), prefix.end(), target) - prefix.begin();
        cuts.push_back(std::max(cuts.back(), std::min(c, n)));
    }
    cuts.push_back(n);
    return cuts;
}

template <typename T>
T* dalloc(size_t count, std::vector<void*>& owned) {
    if (count == 0) count = 1;
    void* p = nullptr;
    ZS_CUDA(cudaMalloc(&p, count * sizeof(T)));
    owned.push_back(p);
    return static_cast<T*>(p);
}

template <typename T>
T* upload(const std::vector<T>& v, std::vector<void*>& owned, cudaStream_t s) {
    T* d = dalloc<T>(v.size(), owned);
    if (!v.empty()) ZS_CUDA(cudaMemcpyAsync(d, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, s));
    return d;
}

}  // namespace

// CUDA-event timing of solve phases (options.profile): event pairs are
// recorded around each phase and folded into the report at every host sync.
struct PhaseTimer {
    bool on = false;
    std::vector<cudaEvent_t> pool;
    std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> pending;
    double ms[8] = {0};
    int calls[8] = {0};
    // nullptr when no event could be created (the phase then goes untimed)
    cudaEvent_t get() noexcept {
        cudaEvent_t e = nullptr;
        if (!pool.empty()) {
            e = pool.back();
            pool.pop_back();
        } else if (cudaEventCreate(&e) != cudaSuccess) {
            cudaGetLastError();
            e = nullptr;
        }
        return e;
    }
    void reset() {
        collect();
        for (int i = 0; i < 8; ++i) ms[i] = 0.0, calls[i] = 0;
    }
    // call only after the stream has been synchronised
    void collect() {
        for (auto& p : pending) {
            float t = 0.f;
            cudaEventElapsedTime(&t, p.second.first, p.second.second);
            ms[p.first] += t;
            calls[p.first] += 1;
            pool.push_back(p.second.first);
            pool.push_back(p.second.second);
        }
        pending.clear();
    }
    void destroy() {
        collect();
        for (cudaEvent_t e : pool) cudaEventDestroy(e);
        pool.clear();
    }
};

struct PhaseScope {
    PhaseTimer& t;
    int phase;
    cudaStream_t s;
    cudaEvent_t e0 = nullptr;
    PhaseScope(PhaseTimer& t_, int ph, cudaStream_t s_) : t(t_), phase(ph), s(s_) {
        if (t.on) {
            e0 = t.get();
            if (e0) cudaEventRecord(e0, s);
        }
    }
    ~PhaseScope() {
        if (t.on && e0) {
            cudaEvent_t e1 = t.get();
            if (!e1) {
                t.pool.push_back(e0);
                return;
            }
            cudaEventRecord(e1, s);
            t.pending.push_back({phase, {e0, e1}});
        }
    }
};

namespace {

// Host scratch of build_problem, kept by the handle across set_problem calls:
// slot i (in call order) grows to the largest size asked for and is not
// cleared between problems, so a repeated problem of similar size touches no
// fresh pages (allocating and zeroing ~150 MB per call cost more than the
// structure analysis itself); it is pinned, so uploads from it are DMA copies.
struct HostScratch {
    std::vector<std::pair<void*, size_t>> slots;
    size_t next = 0;
    void* get(size_t bytes) {
        if (next == slots.size()) slots.push_back({nullptr, 0});
        auto& sl = slots[next++];
        if (sl.second < bytes) {
            if (sl.first) cudaFreeHost(sl.first);
            sl = {nullptr, 0};
            ZS_CUDA(cudaMallocHost(&sl.first, std::max<size_t>(bytes, 1)));
            sl.second = bytes;
        }
        return sl.first;
    }
    void release() {
        for (auto& sl : slots)
            if (sl.first) cudaFreeHost(sl.first);
        slots.clear();
        next = 0;
    }
};

// A view of n elements of scratch (contents undefined until written).
template <typename T>
struct HostArray {
    T* p = nullptr;
    size_t n = 0;
    T& operator[](size_t i) { return p[i]; }
    const T& operator[](size_t i) const { return p[i]; }
    size_t size() const { return n; }
    const T* data() const { return p; }
};

template <typename T>
HostArray<T> scratch_array(HostScratch& hs, size_t n) {
    return HostArray<T>{static_cast<T*>(hs.get(n * sizeof(T))), n};
}

template <typename T>
T* upload(const HostArray<T>& v, DevPool& pool, cudaStream_t s) {
    T* d = dalloc<T>(v.size(), pool);
    if (v.size()) ZS_CUDA(cudaMemcpyAsync(d, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, s));
    return d;
}

}  // namespace

struct zs_ba_handle {
    zs_ba_options opt{};
    PhaseTimer timer;
    int device = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    bool has_problem = false;
    DevProblem P;
    DevWork W;
    LmState* st = nullptr;       // device
    LmState* st_host = nullptr;  // pinned mirror
    DevPool owned;               // problem-lifetime device allocations
    double* adj_rec = nullptr;   // adjoint buffers, allocated on first use (owned)
    double* adj_part = nullptr;
    double* adj_vec = nullptr;   // a, v, r, z, p, q, zero: 7 x (n + 3L)
    double* adj_inv = nullptr;   // L^-1, its transpose and n doubles (n <= kAdjInvMaxN)
    std::vector<int64_t> perm;   // landmark-major position -> caller's observation index
    int tsize = 8;
    HostScratch hscratch;        // build_problem's host arrays (pinned, reused)
    std::vector<zs_ba_attempt> history;  // the last single-problem solve's attempts
    void* aux_buf = nullptr;     // device arrays of map culling and matching (handle lifetime, grown on demand)
    size_t aux_cap = 0;
    // batched windows
    bool batch = false;
    BatchDev B;
    std::vector<int32_t> wpose0, wlm0;  // first pose / landmark of each window, plus the end
    cudaGraph_t bgraph = nullptr;
    cudaGraphExec_t bexec = nullptr;
    int bgraph_iters = -1, bgraph_rel = -1;
    long long bbody_launches = 0, bpro_launches = 0;
    float tune_us[kBatchBuckets] = {0};
    // the blocked preconditioner's streams (mixed form, large n), kept for the
    // handle's lifetime and sized for the largest n seen
    TcStreams tcs;
    int tcs_n = 0;
    // pose-only problems in one launch: free landmarks of the problem, and
    // the launch's report and attempt records (device, handle lifetime)
    int free_landmarks = 0, free_poses = 0;
    PoseOnlyOut* po_out = nullptr;
    zs_ba_attempt* po_hist = nullptr;
    int po_hist_cap = 0;
    double* po_scratch = nullptr;  // partial sums: [grid * 64 * 27] + [64 * 27] + [grid]
    size_t po_scratch_cap = 0;

    void release_graph() {
        if (bexec) cudaGraphExecDestroy(bexec);
        if (bgraph) cudaGraphDestroy(bgraph);
        bexec = nullptr;
        bgraph = nullptr;
        bgraph_iters = bgraph_rel = -1;
    }

    void release_batch_streams() {
        for (int b = 0; b < kBatchBuckets; ++b) {
            if (B.streams[b]) cudaStreamDestroy(B.streams[b]);
            if (B.ev_join[b]) cudaEventDestroy(B.ev_join[b]);
        }
        if (B.ev_fork) cudaEventDestroy(B.ev_fork);
    }

    // keep_memory: the buffers stay for reuse by the next problem
    void release_problem(bool keep_memory = false) {
        release_graph();
        release_batch_streams();
        if (keep_memory) owned.recycle();
        else owned.release_all();
        P = DevProblem{};
        W = DevWork{};
        adj_rec = adj_part = adj_vec = adj_inv = nullptr;
        batch = false;
        B = BatchDev{};
        wpose0.clear();
        wlm0.clear();
        has_problem = false;
    }
};

// Carves the device arrays of map culling and matching out of one handle-owned buffer.
struct Carve {
    char* base;
    size_t off = 0;
    explicit Carve(void* b) : base(static_cast<char*>(b)) {}
    template <typename T>
    T* take(size_t count) {
        T* p = reinterpret_cast<T*>(base + off);
        off += (count * sizeof(T) + 255) & ~size_t(255);
        return p;
    }
    template <typename T>
    static size_t bytes(size_t count) { return (count * sizeof(T) + 255) & ~size_t(255); }
};

static void aux_reserve(zs_ba_handle* h, size_t bytes) {
    if (bytes <= h->aux_cap) return;
    if (h->aux_buf) {
        ZS_CUDA(cudaStreamSynchronize(h->stream));
        ZS_CUDA(cudaFree(h->aux_buf));
        h->aux_buf = nullptr;
        h->aux_cap = 0;
    }
    const size_t cap = std::max(bytes, h->aux_cap + h->aux_cap / 2);
    ZS_CUDA(cudaMalloc(&h->aux_buf, cap));
    h->aux_cap = cap;
}

// Runs k_cull (after `pre`, which enqueues the inputs' copies and any kernel
// they need), copies the outputs back and fills the report.
template <typename Pre, typename Launch>
static int cull_run(zs_ba_handle* h, CullArgs& a, uint8_t* erase, float* mean_error, zs_cull_report* rep,
                    Pre&& pre, Launch&& launch) {
    ZS_CUDA(cudaMemsetAsync(a.counters, 0, 4 * sizeof(unsigned long long), h->stream));
    pre();
    ZS_CUDA(cudaEventRecord(h->ev0, h->stream));
    launch();
    ZS_CUDA(cudaGetLastError());
    ZS_CUDA(cudaEventRecord(h->ev1, h->stream));
    unsigned long long cnt[4] = {0, 0, 0, 0};
    if (erase && a.L > 0)
        ZS_CUDA(cudaMemcpyAsync(erase, a.erase, (size_t)a.L, cudaMemcpyDeviceToHost, h->stream));
    if (mean_error && a.L > 0)
        ZS_CUDA(cudaMemcpyAsync(mean_error, a.mean, sizeof(float) * (size_t)a.L, cudaMemcpyDeviceToHost, h->stream));
    ZS_CUDA(cudaMemcpyAsync(cnt, a.counters, sizeof(cnt), cudaMemcpyDeviceToHost, h->stream));
    ZS_CUDA(cudaStreamSynchronize(h->stream));
    if (cnt[2]) return ZS_ERR_INVALID;
    if (rep) {
        float ms = 0.f;
        ZS_CUDA(cudaEventElapsedTime(&ms, h->ev0, h->ev1));
        rep->erased = (int64_t)cnt[0];
        rep->error_passes = (int64_t)cnt[1];
        rep->ms_device = ms;
    }
    return ZS_OK;
}

extern "C" {

void zs_ba_default_options(zs_ba_options* o) {
    if (!o) return;
    std::memset(o, 0, sizeof(*o));
    o->precision = ZS_PRECISION_FP64;
    o->max_failures = 10;
    o->tau = 1e-5;
    o->diagonal_clamp = 5e10;
    o->legacy_stop = 1e-10;
    o->relative_tolerance = 1e-6;
    o->chi2_floor = 1e-12;
    o->refine_iterations = 8;
    o->refine_tolerance = 1e-10;
    o->device = 0;
    o->verbose = 0;
    o->batch_graph = 1;
    o->autotune_cache = nullptr;
    o->pose_only_path = 1;
}

const char* zs_ba_status_string(int s) {
    switch (s) {
        case ZS_OK: return "ok";
        case ZS_ERR_INVALID: return "invalid argument or problem";
        case ZS_ERR_CUDA: return "CUDA error or no usable CUDA device";
        case ZS_ERR_UNSUPPORTED: return "unsupported vertex, edge or loss kind";
        case ZS_ERR_TIMEOUT: return "a bounded device wait ran out";
        case ZS_ERR_NONFINITE: return "non-finite input values";
        case ZS_ERR_NO_PROBLEM: return "no problem has been set";
        case ZS_ERR_OUT_OF_MEMORY: return "out of device memory";
        case ZS_ERR_CHOLESKY: return "Cholesky solver failed";
        default: return "unknown status";
    }
}

static thread_local char g_last_error[256] = "";

static int cuda_status(cudaError_t e) {
    std::snprintf(g_last_error, sizeof(g_last_error), "%s: %s", cudaGetErrorName(e), cudaGetErrorString(e));
    cudaGetLastError();
    return e == cudaErrorMemoryAllocation ? ZS_ERR_OUT_OF_MEMORY : ZS_ERR_CUDA;
}

const char* zs_last_error(void) { return g_last_error; }

}  // extern "C"

namespace zs {
int record_cuda_error(cudaError_t e) { return cuda_status(e); }
}  // namespace zs

extern "C" {

int zs_ba_create(zs_ba_handle** out, const zs_ba_options* opt) {
    if (!out) return ZS_ERR_INVALID;
    *out = nullptr;
    zs_ba_handle* h = new (std::nothrow) zs_ba_handle();
    if (!h) return ZS_ERR_OUT_OF_MEMORY;
    if (opt) h->opt = *opt;
    else zs_ba_default_options(&h->opt);
    if (h->opt.precision != ZS_PRECISION_FP64 && h->opt.precision != ZS_PRECISION_MIXED) {
        delete h;
        return ZS_ERR_INVALID;
    }
    h->tsize = h->opt.precision == ZS_PRECISION_FP64 ? 8 : 4;
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count <= 0 || h->opt.device < 0 || h->opt.device >= count) {
        cudaGetLastError();
        delete h;
        return ZS_ERR_CUDA;
    }
    h->device = h->opt.device;
    try {
        ZS_CUDA(cudaSetDevice(h->device));
        ZS_CUDA(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
        ZS_CUDA(cudaEventCreate(&h->ev0));
        ZS_CUDA(cudaEventCreate(&h->ev1));
        ZS_CUDA(cudaMalloc(&h->st, sizeof(LmState)));
        ZS_CUDA(cudaMallocHost(&h->st_host, sizeof(LmState)));
        ZS_CUDA(cudaMemset(h->st, 0, sizeof(LmState)));
    } catch (const CudaError& e) {
        zs_ba_destroy(h);
        return cuda_status(e.err);
    }
    *out = h;
    return ZS_OK;
}

void zs_ba_destroy(zs_ba_handle* h) {
    if (!h) return;
    cudaSetDevice(h->device);
    if (h->stream) cudaStreamSynchronize(h->stream);
    h->timer.destroy();
    h->release_problem();
    h->hscratch.release();
    if (h->aux_buf) cudaFree(h->aux_buf);
    if (h->po_out) cudaFree(h->po_out);
    if (h->po_hist) cudaFree(h->po_hist);
    if (h->po_scratch) cudaFree(h->po_scratch);
    if (h->st) cudaFree(h->st);
    if (h->st_host) cudaFreeHost(h->st_host);
    if (h->ev0) cudaEventDestroy(h->ev0);
    if (h->ev1) cudaEventDestroy(h->ev1);
    if (h->stream) cudaStreamDestroy(h->stream);
    delete h;
}

static int validate(const zs_ba_problem* p) {
    if (!p) return ZS_ERR_INVALID;
    if (p->num_poses < 0 || p->num_landmarks < 0 || p->num_obs < 0) return ZS_ERR_INVALID;
    if (p->num_obs > 0x7fffffffLL) return ZS_ERR_INVALID;
    if (p->num_poses > 0 && (!p->poses || !p->pose_fixed)) return ZS_ERR_INVALID;
    if (p->num_landmarks > 0 && (!p->landmarks || !p->landmark_fixed)) return ZS_ERR_INVALID;
    if (p->num_obs > 0 && (!p->obs_pose || !p->obs_landmark || !p->obs_uv)) return ZS_ERR_INVALID;
    if (p->loss_kind < ZS_LOSS_NONE || p->loss_kind > ZS_LOSS_TUKEY) return ZS_ERR_UNSUPPORTED;
    if (p->loss_kind != ZS_LOSS_NONE && !(p->loss_delta > 0.0)) return ZS_ERR_INVALID;
    if (!(p->intrinsics[0] > 0.0) || !(p->intrinsics[1] > 0.0)) return ZS_ERR_INVALID;
    for (int i = 0; i < 4; ++i)
        if (!std::isfinite(p->intrinsics[i])) return ZS_ERR_NONFINITE;
    for (int64_t o = 0; o < p->num_obs; ++o) {
        if (p->obs_pose[o] < 0 || p->obs_pose[o] >= p->num_poses) return ZS_ERR_INVALID;
        if (p->obs_landmark[o] < 0 || p->obs_landmark[o] >= p->num_landmarks) return ZS_ERR_INVALID;
        if (p->obs_info && p->obs_info[4 * o + 1] != p->obs_info[4 * o + 2]) return ZS_ERR_INVALID;
    }
    return ZS_OK;
}

// Builds the device orderings and the Schur pair/triple lists, uploads the
// problem and allocates the working arrays of the handle's precision. With
// windows (wpose0 / wlm0: first pose / landmark of each window, plus the
// end), the problem is a batch of independent windows: pairs stay inside a
// window and S is block diagonal; without, it is one problem.
static void build_problem(zs_ba_handle* h, const zs_ba_problem* p, const std::vector<int32_t>* wpose0 = nullptr,
                          const std::vector<int32_t>* wlm0 = nullptr) {
    cudaStream_t s = h->stream;
    // with options.verbose >= 3: host milliseconds of the steps below
    auto t_prev = std::chrono::steady_clock::now();
    auto stamp = [&](const char* what) {
        if (h->opt.verbose < 3) return;
        const auto t = std::chrono::steady_clock::now();
        std::fprintf(stderr, "  set_problem %-22s %7.2f ms\n", what,
                     std::chrono::duration<double, std::milli>(t - t_prev).count());
        t_prev = t;
    };
    const int K = p->num_poses, L = p->num_landmarks;
    const int64_t M = p->num_obs;
    const bool batched = wpose0 != nullptr;
    const std::vector<int32_t> one_p{0, K}, one_l{0, L};
    const std::vector<int32_t>& wp = batched ? *wpose0 : one_p;
    const std::vector<int32_t>& wl = batched ? *wlm0 : one_l;
    const int nwin = (int)wp.size() - 1;
    DevProblem& P = h->P;
    P.K = K;
    P.L = L;
    P.M = M;
    P.n = 6 * K;
    P.intr = Intrinsics{p->intrinsics[0], p->intrinsics[1], p->intrinsics[2], p->intrinsics[3]};
    P.loss = LossParams{p->loss_kind, p->loss_delta};

    // landmark-major order, poses ascending within a landmark (stable): a
    // parallel counting sort (threads count index ranges per landmark; the
    // landmark totals, then each thread's offsets, by landmark ranges) and a
    // per-landmark sort by pose below
    const int nt = host_threads();
    std::vector<int32_t> lm_ptr(L + 1, 0);
    std::vector<int64_t>& perm = h->perm;
    perm.resize(M);
    {
        const int ntu = (M > 50000 && L > 4 * nt) ? nt : 1;
        std::vector<int64_t> uo(ntu + 1), ul(ntu + 1);
        for (int t = 0; t <= ntu; ++t) {
            uo[t] = M * t / ntu;
            ul[t] = (int64_t)L * t / ntu;
        }
        std::vector<std::vector<int32_t>> cnt(ntu);
        parallel_ranges(uo, [&](int t, int64_t o0, int64_t o1) {
            std::vector<int32_t>& c = cnt[t];
            c.assign(L, 0);
            for (int64_t o = o0; o < o1; ++o) c[p->obs_landmark[o]]++;
        });
        parallel_ranges(ul, [&](int, int64_t l0, int64_t l1) {
            for (int64_t l = l0; l < l1; ++l) {
                int32_t tot = 0;
                for (int t = 0; t < ntu; ++t) tot += cnt[t][l];
                lm_ptr[l + 1] = tot;
            }
        });
        for (int l = 0; l < L; ++l) lm_ptr[l + 1] += lm_ptr[l];
        parallel_ranges(ul, [&](int, int64_t l0, int64_t l1) {
            for (int64_t l = l0; l < l1; ++l) {
                int32_t run = lm_ptr[l];
                for (int t = 0; t < ntu; ++t) {
                    const int32_t c = cnt[t][l];
                    cnt[t][l] = run;  // thread t's first position for landmark l
                    run += c;
                }
            }
        });
        parallel_ranges(uo, [&](int t, int64_t o0, int64_t o1) {
            std::vector<int32_t>& pos = cnt[t];
            for (int64_t o = o0; o < o1; ++o) perm[pos[p->obs_landmark[o]]++] = o;
        });
    }
    // landmark ranges of about equal observation counts
    std::vector<int64_t> obs_prefix(L + 1);
    for (int l = 0; l <= L; ++l) obs_prefix[l] = lm_ptr[l];
    const std::vector<int64_t> lcuts = balanced_cuts(obs_prefix, (M > 50000 && L > 4 * nt) ? nt : 1);
    const int nth = (int)lcuts.size() - 1;
    HostScratch& hs = h->hscratch;
    hs.next = 0;
    HostArray<int32_t> obs_pose = scratch_array<int32_t>(hs, M), obs_lm = scratch_array<int32_t>(hs, M),
                       dup_owner = scratch_array<int32_t>(hs, M);
    HostArray<double2> uv = scratch_array<double2>(hs, M);
    HostArray<double> info = scratch_array<double>(hs, p->obs_info ? 4 * M : 0);
    HostArray<uint8_t> blk_valid = scratch_array<uint8_t>(hs, M);
    std::vector<char> dups(nth, 0);
    parallel_ranges(lcuts, [&](int t, int64_t l0, int64_t l1) {
        for (int64_t l = l0; l < l1; ++l) {
            std::stable_sort(perm.begin() + lm_ptr[l], perm.begin() + lm_ptr[l + 1],
                             [&](int64_t a, int64_t b) { return p->obs_pose[a] < p->obs_pose[b]; });
            for (int64_t i = lm_ptr[l]; i < lm_ptr[l + 1]; ++i) {
                const int64_t o = perm[i];
                obs_pose[i] = p->obs_pose[o];
                obs_lm[i] = p->obs_landmark[o];
                uv[i] = make_double2(p->obs_uv[2 * o], p->obs_uv[2 * o + 1]);
                if (p->obs_info)
                    for (int k = 0; k < 4; ++k) info[4 * i + k] = p->obs_info[4 * o + k];
                const bool same = i > lm_ptr[l] && obs_pose[i - 1] == obs_pose[i];
                dup_owner[i] = same ? dup_owner[i - 1] : (int32_t)i;
                if (same) dups[t] = 1;
                blk_valid[i] = (!same && !p->pose_fixed[obs_pose[i]] && !p->landmark_fixed[obs_lm[i]]) ? 1 : 0;
            }
        }
    });
    bool has_dups = false;
    for (char d : dups) has_dups = has_dups || d;
    stamp("landmark-major order");
    // pose-major lists of landmark-major indices, ascending
    // (a stable counting sort by pose over index ranges of equal length: each
    // thread counts its range per pose and fills after the threads before it)
    // pm: pose-major position of each observation, where its H_pl / W /
    // pose-partial records live, so a pose's records are contiguous
    std::vector<int32_t> pose_ptr(K + 1, 0);
    HostArray<int32_t> pose_obs = scratch_array<int32_t>(hs, M), pm = scratch_array<int32_t>(hs, M);
    {
        std::vector<int64_t> uni(nth + 1);
        for (int t = 0; t <= nth; ++t) uni[t] = M * t / nth;
        std::vector<std::vector<int32_t>> cnt(nth, std::vector<int32_t>(K, 0));
        parallel_ranges(uni, [&](int t, int64_t i0, int64_t i1) {
            for (int64_t i = i0; i < i1; ++i) cnt[t][obs_pose[i]]++;
        });
        for (int k = 0; k < K; ++k) {
            int32_t run = pose_ptr[k];
            for (int t = 0; t < nth; ++t) {
                const int32_t c = cnt[t][k];
                cnt[t][k] = run;  // thread t's first position for pose k
                run += c;
            }
            pose_ptr[k + 1] = run;
        }
        parallel_ranges(uni, [&](int t, int64_t i0, int64_t i1) {
            std::vector<int32_t>& pos = cnt[t];
            for (int64_t i = i0; i < i1; ++i) {
                const int32_t q = pos[obs_pose[i]]++;
                pose_obs[q] = (int32_t)i;
                pm[i] = q;
            }
        });
    }
    // chunks of the mixed form's Schur operator: <= kOpChunk pose-major
    // positions of one pose each
    std::vector<int32_t> opch_q, pose_opch(K + 1, 0);
    for (int k = 0; k < K; ++k) {
        pose_opch[k] = (int32_t)opch_q.size();
        for (int32_t q = pose_ptr[k]; q < pose_ptr[k + 1]; q += kOpChunk) opch_q.push_back(q);
    }
    pose_opch[K] = (int32_t)opch_q.size();
    opch_q.push_back((int32_t)M);
    std::vector<int32_t> lmch_l{0};
    for (int l = 0; l < L; ++l) {
        const int32_t start = lm_ptr[lmch_l.back()];
        if (l > lmch_l.back() && lm_ptr[l + 1] - start > kOpChunk) lmch_l.push_back(l);
    }
    if (lmch_l.back() != L) lmch_l.push_back(L);
    stamp("pose lists, chunks");
    // Schur triples: for each landmark, every (block a, block b) with pose_a >= pose_b,
    // grouped by pose pair (i, j) = (pose_a, pose_b), landmark order within a pair.
    // Pair keys are window-local: key = base_w + (i - p0_w) K_w + (j - p0_w).
    std::vector<int32_t> pose_win(K, 0), lm_win(L, 0);
    std::vector<int64_t> key_base(nwin + 1, 0);
    for (int w = 0; w < nwin; ++w) {
        const int64_t kw = wp[w + 1] - wp[w];
        key_base[w + 1] = key_base[w] + kw * kw;
        for (int k = wp[w]; k < wp[w + 1]; ++k) pose_win[k] = w;
        for (int l = wl[w]; l < wl[w + 1]; ++l) lm_win[l] = w;
    }
    auto pair_key = [&](int i, int j) {
        const int w = pose_win[i];
        const int64_t kw = wp[w + 1] - wp[w];
        return (size_t)(key_base[w] + (int64_t)(i - wp[w]) * kw + (j - wp[w]));
    };
    const size_t nkeys = (size_t)key_base[nwin];
    // Threads take landmark ranges of about equal triple counts; each counts
    // its triples per key, then fills its share of every key's range after the
    // shares of the threads before it, which is the landmark order a single
    // pass would give.
    std::vector<int64_t> tri_prefix(L + 1, 0);
    parallel_ranges(lcuts, [&](int, int64_t l0, int64_t l1) {
        for (int64_t l = l0; l < l1; ++l) {
            int64_t nv = 0;
            for (int32_t i = lm_ptr[l]; i < lm_ptr[l + 1]; ++i) nv += blk_valid[i];
            tri_prefix[l + 1] = nv * (nv + 1) / 2;
        }
    });
    for (int l = 0; l < L; ++l) tri_prefix[l + 1] += tri_prefix[l];
    const int64_t ntriples = tri_prefix[L];
    stamp("triple counts");
    const int ntt = (ntriples > 200000 && L > 4 * nt && (size_t)nt * nkeys <= ((size_t)1 << 28)) ? nt : 1;
    const std::vector<int64_t> tcuts = balanced_cuts(tri_prefix, ntt);
    const int ntc = (int)tcuts.size() - 1;
    std::vector<std::vector<int64_t>> counts(ntc);
    parallel_ranges(tcuts, [&](int t, int64_t l0, int64_t l1) {
        std::vector<int32_t> vb;
        std::vector<int64_t>& c = counts[t];
        c.assign(nkeys, 0);
        for (int64_t l = l0; l < l1; ++l) {
            vb.clear();
            for (int32_t i = lm_ptr[l]; i < lm_ptr[l + 1]; ++i)
                if (blk_valid[i]) vb.push_back(i);
            for (size_t a = 0; a < vb.size(); ++a)
                for (size_t b = 0; b <= a; ++b) c[pair_key(obs_pose[vb[a]], obs_pose[vb[b]])]++;
        }
    });
    // key totals, their prefix, then each thread's first position per key
    // (by key ranges)
    std::vector<int64_t> pair_off(nkeys + 1, 0);
    std::vector<int64_t> pair_count(nkeys, 0);
    std::vector<int64_t> kr(ntc + 1);
    for (int t = 0; t <= ntc; ++t) kr[t] = (int64_t)nkeys * t / ntc;
    parallel_ranges(kr, [&](int, int64_t k0, int64_t k1) {
        for (int64_t k = k0; k < k1; ++k) {
            int64_t tot = 0;
            for (int t = 0; t < ntc; ++t) tot += counts[t][k];
            pair_count[k] = tot;
        }
    });
    int npairs = 0;
    for (size_t k = 0; k < nkeys; ++k) {
        pair_off[k + 1] = pair_off[k] + pair_count[k];
        if (pair_count[k]) ++npairs;
    }
    parallel_ranges(kr, [&](int, int64_t k0, int64_t k1) {
        for (int64_t k = k0; k < k1; ++k) {
            int64_t run = pair_off[k];
            for (int t = 0; t < ntc; ++t) {
                const int64_t c = counts[t][k];
                counts[t][k] = run;  // thread t's first position in key k
                run += c;
            }
        }
    });
    stamp("pair counts");
    HostArray<int2> triples = scratch_array<int2>(hs, ntriples);
    parallel_ranges(tcuts, [&](int t, int64_t l0, int64_t l1) {
        std::vector<int32_t> vb;
        std::vector<int64_t>& pos = counts[t];
        for (int64_t l = l0; l < l1; ++l) {
            vb.clear();
            for (int32_t i = lm_ptr[l]; i < lm_ptr[l + 1]; ++i)
                if (blk_valid[i]) vb.push_back(i);
            for (size_t a = 0; a < vb.size(); ++a)
                for (size_t b = 0; b <= a; ++b)
                    triples[pos[pair_key(obs_pose[vb[a]], obs_pose[vb[b]])]++] = make_int2(pm[vb[a]], pm[vb[b]]);
        }
    });
    counts.clear();
    stamp("triples");
    std::vector<int32_t> pair_i, pair_j, seg_pair;
    std::vector<int64_t> seg_ptr{0}, pair_seg_ptr{0};
    pair_i.reserve(npairs);
    pair_j.reserve(npairs);
    for (int w = 0; w < nwin; ++w) {
        const int64_t kw = wp[w + 1] - wp[w];
        for (int64_t k = key_base[w]; k < key_base[w + 1]; ++k) {
            if (!pair_count[k]) continue;
            pair_i.push_back((int32_t)(wp[w] + (k - key_base[w]) / kw));
            pair_j.push_back((int32_t)(wp[w] + (k - key_base[w]) % kw));
            for (int64_t t = pair_off[k]; t < pair_off[k + 1]; t += kSegment) {
                seg_ptr.push_back(std::min<int64_t>(t + kSegment, pair_off[k + 1]));
                seg_pair.push_back((int32_t)pair_i.size() - 1);
            }
            pair_seg_ptr.push_back((int64_t)seg_pair.size());
        }
    }
    P.npairs = npairs;
    P.ntriples = ntriples;
    P.nsegs = (int64_t)seg_pair.size();
    stamp("segments");

    // state (padded device layout)
    std::vector<double> pose8((size_t)K * kPoseStride, 0.0), lm4((size_t)L * kLmStride, 0.0);
    for (int k = 0; k < K; ++k)
        for (int i = 0; i < 7; ++i) pose8[(size_t)k * kPoseStride + i] = p->poses[7LL * k + i];
    for (int l = 0; l < L; ++l)
        for (int i = 0; i < 3; ++i) lm4[(size_t)l * kLmStride + i] = p->landmarks[3LL * l + i];
    std::vector<uint8_t> pf(p->pose_fixed, p->pose_fixed + K), lf(p->landmark_fixed, p->landmark_fixed + L);
    h->free_landmarks = 0;
    for (int l = 0; l < L; ++l) h->free_landmarks += lf[l] == 0;
    h->free_poses = 0;
    for (int k = 0; k < K; ++k) h->free_poses += pf[k] == 0;

    auto& own = h->owned;
    P.pose = upload(pose8, own, s);
    P.pose_bk = dalloc<double>(pose8.size(), own);
    P.lm = upload(lm4, own, s);
    P.lm_bk = dalloc<double>(lm4.size(), own);
    P.pose_init = upload(pose8, own, s);
    P.lm_init = upload(lm4, own, s);
    P.pose_fixed = upload(pf, own, s);
    P.lm_fixed = upload(lf, own, s);
    P.obs_pose = upload(obs_pose, own, s);
    P.obs_lm = upload(obs_lm, own, s);
    P.obs_uv = upload(uv, own, s);
    P.obs_info = p->obs_info ? upload(info, own, s) : nullptr;
    P.lm_ptr = upload(lm_ptr, own, s);
    P.pose_ptr = upload(pose_ptr, own, s);
    P.pose_obs = upload(pose_obs, own, s);
    P.blk_valid = upload(blk_valid, own, s);
    P.has_dups = has_dups;
    P.dup_owner = has_dups ? upload(dup_owner, own, s) : nullptr;
    P.pair_i = upload(pair_i, own, s);
    P.pair_j = upload(pair_j, own, s);
    P.seg_ptr = upload(seg_ptr, own, s);
    P.seg_pair = upload(seg_pair, own, s);
    P.pair_seg_ptr = upload(pair_seg_ptr, own, s);
    P.pm = upload(pm, own, s);
    P.nopch = (int64_t)opch_q.size() - 1;
    P.opch_q = upload(opch_q, own, s);
    P.pose_opch = upload(pose_opch, own, s);
    P.nlmch = (int64_t)lmch_l.size() - 1;
    P.lmch_l = upload(lmch_l, own, s);
    P.triples = upload(triples, own, s);
    stamp("uploads");
    P.nwin = nwin;
    std::vector<int64_t> win_s_off(nwin, 0);
    int64_t s_total = 0;
    for (int w = 0; w < nwin; ++w) {
        win_s_off[w] = s_total;
        const int64_t nw = 6LL * (wp[w + 1] - wp[w]);
        s_total += nw * nw;
    }
    if (batched) {
        // observation chunks for per-window cost sums, never across windows
        std::vector<int64_t> ochunk_ptr{0};
        std::vector<int32_t> ochunk_win, win_ochunk{0};
        for (int w = 0; w < nwin; ++w) {
            const int64_t o0 = lm_ptr[wl[w]], o1 = lm_ptr[wl[w + 1]];
            for (int64_t o = o0; o < o1; o += kBatchObsChunk) {
                ochunk_ptr.push_back(std::min<int64_t>(o + kBatchObsChunk, o1));
                ochunk_win.push_back(w);
            }
            win_ochunk.push_back((int32_t)ochunk_win.size());
        }
        P.nochunks = (int64_t)ochunk_win.size();
        P.pose_win = upload(pose_win, own, s);
        P.lm_win = upload(lm_win, own, s);
        P.win_pose0 = upload(wp, own, s);
        P.win_lm0 = upload(wl, own, s);
        P.win_s_off = upload(win_s_off, own, s);
        P.ochunk_ptr = upload(ochunk_ptr, own, s);
        P.ochunk_win = upload(ochunk_win, own, s);
        P.win_ochunk = upload(win_ochunk, own, s);
    }

    const size_t ts = (size_t)h->tsize;
    const int n = P.n;
    DevWork& W = h->W;
    const size_t rs = h->tsize == 4 ? 20 : 18;  // padded H_pl / W record
    W.hpl = dalloc<char>(ts * rs * M, own);
    W.W = dalloc<char>(ts * rs * M, own);
    W.pose_aux = dalloc<double>((size_t)K * 24, own);
    W.partial = dalloc<double>(36 * (size_t)P.nsegs, own);
    W.opch_sum = dalloc<double>(6 * (size_t)std::max<int64_t>(P.nopch, 1), own);
    if (h->tsize == 4) {
        W.jac = dalloc<ObsJac>((size_t)M, own);
        W.jp_pm = dalloc<float4>(3 * (size_t)M, own);
        W.hll_inv_f = dalloc<float>(12 * (size_t)std::max(L, 1), own);
    }
    else W.lm_part = dalloc<char>(ts * 12 * M, own);  // record-major, 9 values padded to 12
    W.pose_part = dalloc<char>(ts * 28 * M, own);  // record-major, 27 values padded to 28
    W.hpp = dalloc<double>((size_t)K * 36, own);
    W.hll = dalloc<double>((size_t)L * 9, own);
    W.hll_inv = dalloc<double>((size_t)L * 9, own);
    W.b = dalloc<double>((size_t)n + 3 * (size_t)L, own);
    W.S = dalloc<double>((size_t)s_total, own);
    W.bs = dalloc<double>(n, own);
    if (!batched) {
        W.F = dalloc<char>(ts * (size_t)n * n, own);
        W.D = dalloc<char>(ts * 1024 * (size_t)((n + 31) / 32), own);
        W.work = dalloc<double>(4 * (size_t)n + 256, own);
        if (h->tsize == 4) {
            W.X = dalloc<char>(ts * (size_t)n * n, own);
            W.XT = dalloc<char>(ts * (size_t)n * n, own);
            W.pcg = dalloc<double>(pcg_doubles(P), own);
            if (chol_tc_applies(n)) {
                W.tc_scratch = dalloc<float>((size_t)chol_tc_scratch_floats(n), own);
                if (h->tcs_n < n) {
                    ZS_CUDA(h->tcs.init(n));
                    h->tcs_n = n;
                }
                W.tc_streams = &h->tcs;
            }
            W.dag_flags = dalloc<int>((size_t)dag_flag_ints(n), own);
            W.dag_epoch = 0;
            ZS_CUDA(cudaMemsetAsync(W.dag_flags, 0, sizeof(int) * (size_t)dag_flag_ints(n), s));
        }
    }
    W.delta = dalloc<double>((size_t)n + 3 * (size_t)L, own);
    // (+16: the adjoint loop's device scalars, AdjCg, after the partial sums)
    W.red = dalloc<double>(std::max<size_t>(kReduceBlocks * 4 + 16, (size_t)P.nochunks), own);
    W.ired = dalloc<int32_t>(kReduceBlocks, own);
    ZS_CUDA(cudaMemsetAsync(W.hll_inv, 0, sizeof(double) * 9 * (size_t)std::max(L, 1), s));
    ZS_CUDA(cudaMemsetAsync(W.delta, 0, sizeof(double) * std::max<size_t>(1, (size_t)n + 3 * (size_t)L), s));
    ZS_CUDA(cudaStreamSynchronize(s));
    ZS_CUDA(cudaGetLastError());
    stamp("allocations, sync");
}

int zs_ba_set_problem(zs_ba_handle* h, const zs_ba_problem* p) {
    if (!h) return ZS_ERR_INVALID;
    const int v = validate(p);
    if (v != ZS_OK) return v;
    try {
        ZS_CUDA(cudaSetDevice(h->device));
        ZS_CUDA(cudaStreamSynchronize(h->stream));
        h->release_problem(true);
        build_problem(h, p);
        h->owned.trim();
        h->has_problem = true;
    } catch (const CudaError& e) {
        h->release_problem();
        return cuda_status(e.err);
    } catch (const std::bad_alloc&) {
        h->release_problem();
        return ZS_ERR_OUT_OF_MEMORY;
    }
    return ZS_OK;
}

int zs_ba_set_state(zs_ba_handle* h, const double* poses, const double* landmarks) {
    if (!h) return ZS_ERR_INVALID;
    if (!h->has_problem) return ZS_ERR_NO_PROBLEM;
    const DevProblem& P = h->P;
    try {
        ZS_CUDA(cudaSetDevice(h->device));
        if (poses && P.K > 0) {
            ZS_CUDA(cudaMemcpy2DAsync(P.pose, kPoseStride * sizeof(double), poses, 7 * sizeof(double),
                                      7 * sizeof(double), P.K, cudaMemcpyHostToDevice, h->stream));
        }
        if (landmarks && P.L > 0) {
            ZS_CUDA(cudaMemcpy2DAsync(P.lm, kLmStride * sizeof(double), landmarks, 3 * sizeof(double),
                                      3 * sizeof(double), P.L, cudaMemcpyHostToDevice, h->stream));
        }
        ZS_CUDA(cudaStreamSynchronize(h->stream));
    } catch (const CudaError& e) {
        return cuda_status(e.err);
    }
    return ZS_OK;
}

int zs_ba_get_state(zs_ba_handle* h, double* poses, double* landmarks) {
    if (!h) return ZS_ERR_INVALID;
    if (!h->has_problem) return ZS_ERR_NO_PROBLEM;
    const DevProblem& P = h->P;
    try {
        ZS_CUDA(cudaSetDevice(h->device));
        if (poses && P.K > 0) {
            ZS_CUDA(cudaMemcpy2DAsync(poses, 7 * sizeof(double), P.pose, kPoseStride * sizeof(double),
                                      7 * sizeof(double), P.K, cudaMemcpyDeviceToHost, h->stream));
        }
        if (landmarks && P.L > 0) {
            ZS_CUDA(cudaMemcpy2DAsync(landmarks, 3 * sizeof(double), P.lm, kLmStride * sizeof(double),
                                      3 * sizeof(double), P.L, cudaMemcpyDeviceToHost, h->stream));
        }
        ZS_CUDA(cudaStreamSynchronize(h->stream));
    } catch (const CudaError& e) {
        return cuda_status(e.err);
    }
    return ZS_OK;
}

int zs_ba_reset_state(zs_ba_handle* h) {
    if (!h) return ZS_ERR_INVALID;
    if (!h->has_problem) return ZS_ERR_NO_PROBLEM;
    const DevProblem& P = h->P;
    try {
        ZS_CUDA(cudaSetDevice(h->device));
        if (P.K > 0)
            ZS_CUDA(cudaMemcpyAsync(P.pose, P.pose_init, sizeof(double) * kPoseStride * (size_t)P.K,
                                    cudaMemcpyDeviceToDevice, h->stream));
        if (P.L > 0)
            ZS_CUDA(cudaMemcpyAsync(P.lm, P.lm_init, sizeof(double) * kLmStride * (size_t)P.L,
                                    cudaMemcpyDeviceToDevice, h->stream));
        ZS_CUDA(cudaStreamSynchronize(h->stream));
    } catch (const CudaError& e) {
        return cuda_status(e.err);
    }
    return ZS_OK;
}

}  // extern "C"

namespace {

void read_state(zs_ba_handle* h) {
    ZS_CUDA(cudaMemcpyAsync(h->st_host, h->st, sizeof(LmState), cudaMemcpyDeviceToHost, h->stream));
    ZS_CUDA(cudaStreamSynchronize(h->stream));
    if (h->timer.on) h->timer.collect();
}

template <typename T>
void linearize(zs_ba_handle* h) {
    PhaseScope ps(h->timer, ZS_PHASE_LINEARIZE, h->stream);
    launch_linearize<T>(h->P, h->W, h->stream);
}

// Mixed form: relative diagonal shift of the preconditioner's retry
// factorisation (S + mu diag(S)) after the FP32 factorisation of the
// FP32-formed S failed.
constexpr double kPreconditionerShift = 1e-5;

// One damped solve at st->lambda: H_ll inverses, Schur complement, reduced
// Cholesky solve into delta[0..n), landmark back-substitution.
template <typename T>
void system_solve(zs_ba_handle* h) {
    DevProblem& P = h->P;
    DevWork& W = h->W;
    cudaStream_t s = h->stream;
    launch_set_solve_ok(h->st, 1, s);
    {
        PhaseScope ps(h->timer, ZS_PHASE_INVERT, s);
        launch_invert_w<T>(P, W, h->st, s);
    }
    {
        PhaseScope ps(h->timer, ZS_PHASE_SCHUR, s);
        launch_schur<T>(P, W, h->st, s);
    }
    {
        PhaseScope ps(h->timer, ZS_PHASE_FACTOR, s);
        if constexpr (sizeof(T) == 4)  // the conjugate-gradient preconditioner: L and X = L^-1
            ZS_CUDA(launch_preconditioner(P.n, W.S, (float*)W.F, (float*)W.X, (float*)W.XT, W.tc_scratch,
                                          W.tc_streams, h->st, kPreconditionerShift, W.dag_flags, &W.dag_epoch, s));
        else
            ZS_CUDA((launch_factor<double, T>(P.n, W.S, (T*)W.F, (T*)W.D, h->st, s)));
    }
    {
        PhaseScope ps(h->timer, ZS_PHASE_TRISOLVE, s);
        if constexpr (sizeof(T) == 4) {
            // mixed form: conjugate gradients on the FP64 Schur operator
            // preconditioned by X^T X; it also writes b_s and the landmark
            // back-substitution
            ZS_CUDA(launch_pcg(P, W, h->st, std::max(0, h->opt.refine_iterations), h->opt.refine_tolerance, s));
        } else {
            ZS_CUDA((launch_solve_refine<double, double>(P.n, W.S, (const double*)W.F, (const double*)W.D, W.bs,
                                                         W.delta, W.work, h->st, 0, 0.0, s)));
        }
    }
    if constexpr (sizeof(T) == 8) {
        PhaseScope ps(h->timer, ZS_PHASE_UPDATE, s);
        launch_backsub<T>(P, W, h->st, s);
    }
}

template <typename T>
int solve_impl(zs_ba_handle* h, int iterations, bool use_relative, zs_ba_report* rep) {
    DevProblem& P = h->P;
    DevWork& W = h->W;
    cudaStream_t s = h->stream;
    const zs_ba_options& o = h->opt;
    zs_ba_report r{};
    const long long launches0 = launch_counter();
    h->timer.on = o.profile != 0;
    h->timer.reset();
    ZS_CUDA(cudaEventRecord(h->ev0, s));
    linearize<T>(h);
    {
        PhaseScope ps(h->timer, ZS_PHASE_COST, s);
        if (sizeof(T) == 4) launch_cost_fast(P, W, h->st, false, s);
        else launch_cost(P, W, h->st, false, s);
        launch_init_lambda(P, W, h->st, o.tau, o.diagonal_clamp, s);
    }
    read_state(h);
    LmState& hs = *h->st_host;
    r.chi2_initial = hs.chi2;
    double chi2 = hs.chi2;
    double lambda = hs.lambda;
    if (o.verbose)
        std::fprintf(stderr,
                     "[INIT] iter: XXX, attempt XXX, chi = % 7.7f, rho = XXXX.XXXXXXX, base lambda = % 8.7f\n", chi2,
                     lambda);
    const double legacy = o.legacy_stop * chi2;
    int success = 0;
    h->history.clear();
    for (int it = 0; it < iterations; ++it) {
        r.iterations = it + 1;
        const double last = chi2;
        int failures = 0;
        while (failures < o.max_failures) {
            system_solve<T>(h);
            {
                PhaseScope ps(h->timer, ZS_PHASE_UPDATE, s);
                launch_update(P, W, h->st, s);
                launch_scale(P, W, h->st, s);
            }
            {
                PhaseScope ps(h->timer, ZS_PHASE_COST, s);
                if (sizeof(T) == 4) launch_cost_fast(P, W, h->st, true, s);
                else launch_cost(P, W, h->st, true, s);
                launch_decide(h->st, s);
                launch_rollback(P, h->st, s);
            }
            read_state(h);
            r.attempts++;
            if (hs.timeout) {  // a bounded device wait ran out: the solve stops with the state restored
                std::snprintf(g_last_error, sizeof(g_last_error), "a dependency wait of the preconditioner ran out");
                r.status = ZS_ERR_TIMEOUT;
                if (rep) *rep = r;
                return ZS_ERR_TIMEOUT;
            }
            lambda = hs.lambda;
            {
                zs_ba_attempt a{};
                a.iteration = it;
                a.attempt = failures;
                a.solved = hs.solve_ok ? 1 : 0;
                a.accepted = hs.solve_ok && hs.good ? 1 : 0;
                a.chi2 = hs.solve_ok ? hs.chi2_new : chi2;
                a.rho = hs.solve_ok ? hs.rho : 0.0;
                a.lambda = lambda;
                h->history.push_back(a);
            }
            if (!hs.solve_ok) {
                r.cholesky_failures++;
                if (sizeof(T) == 4) r.preconditioner_retries += hs.shifted;
                if (o.verbose) std::fprintf(stderr, "Cholesky solver failed!\n");
                ++failures;
                if (!std::isfinite(lambda)) break;
                continue;
            }
            if (sizeof(T) == 4) {
                r.refine_sweeps += hs.refine_sweeps;
                r.preconditioner_retries += hs.shifted;
                if (o.verbose > 1)
                    std::fprintf(stderr, "  refinement: %d sweeps, |b - S x| / |b| = %.3e%s\n", hs.refine_sweeps,
                                 hs.rhs_norm > 0.0 ? hs.resid_norm / hs.rhs_norm : 0.0,
                                 hs.shifted ? ", preconditioner shifted" : "");
            }
            if (hs.good) {
                chi2 = hs.chi2;
                ++success;
                if (o.verbose)
                    std::fprintf(stderr,
                                 "[GOOD] iter: % 3d, attempt % 3d, chi2 = % 7.7f, rho = % 7.7f, next lambda = % 8.7f\n",
                                 it, failures, hs.chi2_new, hs.rho, lambda);
                if (!std::isfinite(lambda)) break;
                linearize<T>(h);
                break;
            }
            if (o.verbose)
                std::fprintf(stderr,
                             "[ BAD] iter: % 3d, attempt % 3d, chi2 = % 7.7f, rho = % 7.7f, next lambda = % 8.7f\n", it,
                             failures, hs.chi2_new, hs.rho, lambda);
            if (!std::isfinite(lambda)) break;
            ++failures;
        }
        const double thr = use_relative ? o.relative_tolerance * std::max(last, o.chi2_floor) : legacy;
        if (failures >= o.max_failures || (last - chi2) < thr || !std::isfinite(lambda)) break;
    }
    ZS_CUDA(cudaEventRecord(h->ev1, s));
    ZS_CUDA(cudaEventSynchronize(h->ev1));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, h->ev0, h->ev1);
    r.ms_total = ms;
    r.kernel_launches = launch_counter() - launches0;
    if (h->timer.on) {
        h->timer.collect();
        for (int i = 0; i < 8; ++i) {
            r.ms_phase[i] = h->timer.ms[i];
            r.phase_calls[i] = h->timer.calls[i];
        }
        h->timer.on = false;
    }
    r.accepted = success;
    r.chi2_final = chi2;
    r.lambda_final = lambda;
    r.status = ZS_OK;
    if (rep) *rep = r;
    return success;
}

template <typename T>
int linear_step_impl(zs_ba_handle* h, double lambda, double* S, double* bs, double* delta, double* b) {
    DevProblem& P = h->P;
    DevWork& W = h->W;
    cudaStream_t s = h->stream;
    linearize<T>(h);
    LmState init{};
    init.lambda = lambda;
    init.nu = 2.0;
    ZS_CUDA(cudaMemcpyAsync(h->st, &init, sizeof(LmState), cudaMemcpyHostToDevice, s));
    system_solve<T>(h);
    read_state(h);
    const int n = P.n;
    const size_t nall = (size_t)n + 3 * (size_t)P.L;
    if (S && n > 0) ZS_CUDA(cudaMemcpyAsync(S, W.S, (size_t)n * n * sizeof(double), cudaMemcpyDeviceToHost, s));
    if (bs && n > 0) ZS_CUDA(cudaMemcpyAsync(bs, W.bs, n * sizeof(double), cudaMemcpyDeviceToHost, s));
    if (delta && nall > 0) ZS_CUDA(cudaMemcpyAsync(delta, W.delta, nall * sizeof(double), cudaMemcpyDeviceToHost, s));
    if (b && nall > 0) ZS_CUDA(cudaMemcpyAsync(b, W.b, nall * sizeof(double), cudaMemcpyDeviceToHost, s));
    ZS_CUDA(cudaStreamSynchronize(s));
    if (h->st_host->timeout) return ZS_ERR_TIMEOUT;
    return h->st_host->solve_ok ? ZS_OK : ZS_ERR_CHOLESKY;
}

// The mixed form under Tukey's redescending loss is not offered: its FP32
// Jacobian moves the step by ~1e-5 relative, which moves observations across
// the loss's threshold (weight 0 beyond it) within a few iterations, and the
// solve then settles in a different nearby minimum than the FP64 one (about
// 4e-3 relative in cost after five iterations on a 10-keyframe arc) instead of
// meeting the mixed form's 1e-6 agreement.
bool mixed_tukey(const zs_ba_handle* h) { return h->tsize == 4 && h->P.loss.kind == ZS_LOSS_TUKEY; }

// A single problem whose landmarks are all fixed, with at most
// kPoseOnlyMaxK poses of which at most kPoseOnlyMaxFree free: the pose-only
// path (ba_pose_only.cu).
bool pose_only(const zs_ba_handle* h) {
    return h->opt.pose_only_path != 0 && !h->batch && h->free_landmarks == 0 && h->P.K <= kPoseOnlyMaxK &&
           h->free_poses <= kPoseOnlyMaxFree;
}

// A batch whose landmarks are all fixed (every window at most
// ZS_BATCH_MAX_POSES <= kPoseOnlyMaxK poses): one CTA per window
// (k_pose_only_windows).
bool pose_only_batch(const zs_ba_handle* h) {
    return h->opt.pose_only_path != 0 && h->batch && h->free_landmarks == 0;
}

int pose_only_solve(zs_ba_handle* h, int iterations, bool use_relative, zs_ba_report* rep) {
    cudaStream_t s = h->stream;
    const zs_ba_options& o = h->opt;
    const long long launches0 = launch_counter();
    const int cap = std::max(1, iterations * std::max(1, o.max_failures));
    if (!h->po_out) ZS_CUDA(cudaMalloc(&h->po_out, sizeof(PoseOnlyOut)));
    if (h->po_hist_cap < cap) {
        if (h->po_hist) ZS_CUDA(cudaFree(h->po_hist));
        h->po_hist = nullptr;
        h->po_hist_cap = 0;
        ZS_CUDA(cudaMalloc(&h->po_hist, sizeof(zs_ba_attempt) * (size_t)cap));
        h->po_hist_cap = cap;
    }
    const int grid = pose_only_grid(h->P.M);
    const size_t need = (size_t)grid * kPoseOnlyMaxK * 27 + (size_t)kPoseOnlyMaxK * 27 + (size_t)grid;
    if (h->po_scratch_cap < need) {
        if (h->po_scratch) ZS_CUDA(cudaFree(h->po_scratch));
        h->po_scratch = nullptr;
        h->po_scratch_cap = 0;
        ZS_CUDA(cudaMalloc(&h->po_scratch, sizeof(double) * need));
        h->po_scratch_cap = need;
    }
    double* part = h->po_scratch;
    double* sums = part + (size_t)grid * kPoseOnlyMaxK * 27;
    double* cpart = sums + (size_t)kPoseOnlyMaxK * 27;
    PoseOnlyCtl ctl{o.tau, o.diagonal_clamp, o.legacy_stop, o.relative_tolerance, o.chi2_floor,
                    o.max_failures, iterations, use_relative ? 1 : 0, h->po_hist_cap};
    ZS_CUDA(cudaEventRecord(h->ev0, s));
    ZS_CUDA(launch_pose_only_lm(h->P, ctl, h->po_out, h->po_hist, part, sums, cpart, grid, s));
    ZS_CUDA(cudaEventRecord(h->ev1, s));
    PoseOnlyOut out{};
    ZS_CUDA(cudaMemcpyAsync(&out, h->po_out, sizeof(out), cudaMemcpyDeviceToHost, s));
    ZS_CUDA(cudaStreamSynchronize(s));
    const int nh = std::min(out.history, h->po_hist_cap);
    h->history.assign((size_t)nh, zs_ba_attempt{});
    if (nh > 0)
        ZS_CUDA(cudaMemcpy(h->history.data(), h->po_hist, sizeof(zs_ba_attempt) * (size_t)nh,
                           cudaMemcpyDeviceToHost));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, h->ev0, h->ev1);
    zs_ba_report r{};
    r.status = ZS_OK;
    r.iterations = out.iterations;
    r.accepted = out.accepted;
    r.attempts = out.attempts;
    r.cholesky_failures = out.cholesky_failures;
    r.chi2_initial = out.chi2_initial;
    r.chi2_final = out.chi2_final;
    r.lambda_final = out.lambda_final;
    r.ms_total = ms;
    r.kernel_launches = launch_counter() - launches0;
    if (o.verbose)
        for (const zs_ba_attempt& a : h->history)
            std::fprintf(stderr, "[%s] iter: % 3d, attempt % 3d, chi2 = % 7.7f, rho = % 7.7f, next lambda = % 8.7f\n",
                         a.accepted ? "GOOD" : (a.solved ? " BAD" : "FAIL"), a.iteration, a.attempt, a.chi2, a.rho,
                         a.lambda);
    if (rep) *rep = r;
    return out.accepted;
}

}  // namespace

extern "C" {

int zs_ba_solve(zs_ba_handle* h, int iterations, int use_relative, zs_ba_report* rep) {
    if (!h) return ZS_ERR_INVALID;
    if (rep) std::memset(rep, 0, sizeof(*rep));
    if (!h->has_problem) return ZS_ERR_NO_PROBLEM;
    if (h->batch) return ZS_ERR_UNSUPPORTED;  // zs_ba_solve_batch
    if (mixed_tukey(h) && !pose_only(h)) return ZS_ERR_UNSUPPORTED;
    // source/factor_graph.hpp:494-499: nothing to do without edges or vertices
    if (h->P.M == 0 || (h->P.K == 0 && h->P.L == 0)) return 0;
    if (iterations < 0) return ZS_ERR_INVALID;
    try {
        ZS_CUDA(cudaSetDevice(h->device));
        if (pose_only(h)) {
            const int v = pose_only_solve(h, iterations, use_relative != 0, rep);
            ZS_CUDA(cudaGetLastError());
            return v;
        }
        const int v = h->tsize == 8 ? solve_impl<double>(h, iterations, use_relative != 0, rep)
                                    : solve_impl<float>(h, iterations, use_relative != 0, rep);
        ZS_CUDA(cudaGetLastError());
        return v;
    } catch (const CudaError& e) {
        const int st = cuda_status(e.err);
        if (rep) rep->status = st;
        return st;
    }
}

int zs_ba_chi2(zs_ba_handle* h, double* chi2) {
    if (!h || !chi2) return ZS_ERR_INVALID;
    if (!h->has_problem) return ZS_ERR_NO_PROBLEM;
    try {
        ZS_CUDA(cudaSetDevice(h->device));
        if (h->P.M == 0) {
            *chi2 = 0.0;
            return ZS_OK;
        }
        launch_cost(h->P, h->W, h->st, false, h->stream);
        read_state(h);
        *chi2 = h->st_host->chi2_new;
    } catch (const CudaError& e) {
        return cuda_status(e.err);
    }
    return ZS_OK;
}

int zs_ba_initial_lambda(zs_ba_handle* h, double* lambda) {
    if (!h || !lambda) return ZS_ERR_INVALID;
    if (!h->has_problem) return ZS_ERR_NO_PROBLEM;
    try {
        ZS_CUDA(cudaSetDevice(h->device));
        if (h->tsize == 8) linearize<double>(h);
        else linearize<float>(h);
        launch_cost(h->P, h->W, h->st, false, h->stream);
        launch_init_lambda(h->P, h->W, h->st, h->opt.tau, h->opt.diagonal_clamp, h->stream);
        read_state(h);
        *lambda = h->st_host->lambda;
    } catch (const CudaError& e) {
        return cuda_status(e.err);
    }
    return ZS_OK;
}

int zs_find_matches(zs_ba_handle* h, const uint8_t* lhs, int64_t lhs_count, const uint8_t* rhs, int64_t rhs_count,
                    float threshold, int64_t matches_count, zs_match* matches, int64_t matches_size, int64_t* found,
                    double* ms_device) {
    if (!h || !found) return ZS_ERR_INVALID;
    *found = 0;
    if (ms_device) *ms_device = 0.0;
    if (matches_count <= 0 || matches_size <= 0) return ZS_OK;  // feature.hpp:1200-1202
    if (!matches || lhs_count < 0 || rhs_count < 0) return ZS_ERR_INVALID;
    if (lhs_count > 0x3fffffff || rhs_count > 0x3fffffff) return ZS_ERR_INVALID;
    if ((lhs_count > 0 && !lhs) || (rhs_count > 0 && !rhs)) return ZS_ERR_INVALID;
    if (matches_count > ZS_MATCH_MAX_K) return ZS_ERR_UNSUPPORTED;
    if (lhs_count == 0) return ZS_OK;
    const int nl = (int)lhs_count, nr = (int)rhs_count, k = (int)matches_count;
    // a distance d is kept when (float)d < threshold
    int d_lim = 257;
    for (int d = 0; d <= 256; ++d)
        if (!((float)d < threshold)) {
            d_lim = d;
            break;
        }
    try {
        ZS_CUDA(cudaSetDevice(h->device));
        const int chunks = match_chunks(nl, nr);
        using C = Carve;
        aux_reserve(h, C::bytes<uint8_t>(32 * (size_t)nl) + C::bytes<uint8_t>(32 * (size_t)nr) +
                           C::bytes<unsigned long long>(chunks > 1 ? (size_t)chunks * nl * k : 1) +
                           C::bytes<unsigned long long>((size_t)nl * k));
        C c(h->aux_buf);
        uint8_t* dl = c.take<uint8_t>(32 * (size_t)nl);
        uint8_t* dr = c.take<uint8_t>(32 * (size_t)nr);
        unsigned long long* part = c.take<unsigned long long>(chunks > 1 ? (size_t)chunks * nl * k : 1);
        unsigned long long* out = c.take<unsigned long long>((size_t)nl * k);
        ZS_CUDA(cudaMemcpyAsync(dl, lhs, 32 * (size_t)nl, cudaMemcpyHostToDevice, h->stream));
        if (nr > 0) ZS_CUDA(cudaMemcpyAsync(dr, rhs, 32 * (size_t)nr, cudaMemcpyHostToDevice, h->stream));
        ZS_CUDA(cudaEventRecord(h->ev0, h->stream));
        launch_match(dl, nl, dr, nr, k, d_lim, chunks, part, out, h->stream);
        ZS_CUDA(cudaGetLastError());
        ZS_CUDA(cudaEventRecord(h->ev1, h->stream));
        std::vector<unsigned long long> keys((size_t)nl * k);
        ZS_CUDA(cudaMemcpyAsync(keys.data(), out, sizeof(unsigned long long) * keys.size(), cudaMemcpyDeviceToHost,
                                h->stream));
        ZS_CUDA(cudaStreamSynchronize(h->stream));
        if (ms_device) {
            float ms = 0.f;
            ZS_CUDA(cudaEventElapsedTime(&ms, h->ev0, h->ev1));
            *ms_device = ms;
        }
        // the reference's layout, feature.hpp:1204-1232
        int64_t count = 0;
        for (int i = 0; i < nl; ++i) {
            if (count + k > matches_size) break;
            for (int m = 0; m < k; ++m) {
                const unsigned long long key = keys[(size_t)i * k + m];
                if (key == ~0ull) break;
                zs_match& o = matches[count++];
                o.lhs_index = (uint64_t)i;
                o.rhs_index = (uint64_t)(key & 0xffffffffull);
                o.score = (float)(unsigned int)(key >> 32);
            }
        }
        *found = count;
    } catch (const CudaError& e) {
        return cuda_status(e.err);
    }
    return ZS_OK;
}

int zs_map_cull(zs_ba_handle* h, const zs_map_cull_input* in, uint8_t* erase, float* mean_error,
                zs_cull_report* rep) {
    if (!h || !in) return ZS_ERR_INVALID;
    const int F = in->num_frames, L = in->num_landmarks;
    if (F < 0 || L < 0) return ZS_ERR_INVALID;
    if (L > 0 && (!in->landmark_id || !in->landmarks || !in->landmark_obs)) return ZS_ERR_INVALID;
    if (F > 0 && (!in->frame_pose || !in->frame_intrinsics)) return ZS_ERR_INVALID;
    const int64_t M = L > 0 ? in->landmark_obs[L] : 0;
    if (L > 0 && (in->landmark_obs[0] != 0 || M < 0)) return ZS_ERR_INVALID;
    if (M > 0 && (!in->obs_frame || !in->obs_frame_id || !in->obs_keypoint)) return ZS_ERR_INVALID;
    try {
        ZS_CUDA(cudaSetDevice(h->device));
        using C = Carve;
        aux_reserve(h, C::bytes<unsigned long long>(4) + C::bytes<double>(12 * (size_t)F) +
                            C::bytes<double>(4 * (size_t)F) + C::bytes<int32_t>(L) + C::bytes<double>(3 * (size_t)L) +
                            C::bytes<int64_t>((size_t)L + 1) + 2 * C::bytes<int32_t>((size_t)M) +
                            C::bytes<float2>((size_t)M) + C::bytes<uint8_t>(L) + C::bytes<float>(L));
        C c(h->aux_buf);
        CullArgs a;
        a.L = L;
        a.F = F;
        a.M = M;
        a.counters = c.take<unsigned long long>(4);
        double* Rt = c.take<double>(12 * (size_t)F);
        double* intr = c.take<double>(4 * (size_t)F);
        int32_t* lm_id = c.take<int32_t>(L);
        double* lm = c.take<double>(3 * (size_t)L);
        int64_t* obs_ptr = c.take<int64_t>((size_t)L + 1);
        int32_t* obs_frame = c.take<int32_t>((size_t)M);
        int32_t* obs_frame_id = c.take<int32_t>((size_t)M);
        float2* kp = c.take<float2>((size_t)M);
        a.erase = c.take<uint8_t>(L);
        a.mean = c.take<float>(L);
        a.Rt = Rt;
        a.intr = intr;
        a.intr_stride = 4;
        a.lm = lm;
        a.lm_stride = 3;
        a.lm_id = lm_id;
        a.obs_frame = obs_frame;
        a.obs_frame_id = obs_frame_id;
        a.lm_gen = in->landmark_id_generator;
        a.frame_gen = in->frame_id_generator;
        auto h2d = [&](void* d, const void* src, size_t bytes) {
            if (bytes) ZS_CUDA(cudaMemcpyAsync(d, src, bytes, cudaMemcpyHostToDevice, h->stream));
        };
        return cull_run(h, a, erase, mean_error, rep, [&] {
            h2d(Rt, in->frame_pose, sizeof(double) * 12 * (size_t)F);
            h2d(intr, in->frame_intrinsics, sizeof(double) * 4 * (size_t)F);
            h2d(lm_id, in->landmark_id, sizeof(int32_t) * (size_t)L);
            h2d(lm, in->landmarks, sizeof(double) * 3 * (size_t)L);
            if (L > 0) h2d(obs_ptr, in->landmark_obs, sizeof(int64_t) * ((size_t)L + 1));
            h2d(obs_frame, in->obs_frame, sizeof(int32_t) * (size_t)M);
            h2d(obs_frame_id, in->obs_frame_id, sizeof(int32_t) * (size_t)M);
            h2d(kp, in->obs_keypoint, sizeof(float2) * (size_t)M);
        }, [&] { launch_cull(a, obs_ptr, kp, h->stream); });
    } catch (const CudaError& e) {
        return cuda_status(e.err);
    }
}

int zs_ba_cull(zs_ba_handle* h, const int32_t* landmark_id, const int32_t* pose_frame_id,
               int32_t landmark_id_generator, int32_t frame_id_generator, uint8_t* erase, float* mean_error,
               zs_cull_report* rep) {
    if (!h) return ZS_ERR_INVALID;
    if (!h->has_problem) return ZS_ERR_NO_PROBLEM;
    if (h->batch) return ZS_ERR_UNSUPPORTED;
    const DevProblem& P = h->P;
    if ((P.L > 0 && !landmark_id) || (P.K > 0 && !pose_frame_id)) return ZS_ERR_INVALID;
    try {
        ZS_CUDA(cudaSetDevice(h->device));
        using C = Carve;
        aux_reserve(h, C::bytes<unsigned long long>(4) + C::bytes<double>(12 * (size_t)P.K) +
                            C::bytes<double>(4) + C::bytes<int32_t>(P.L) + C::bytes<int32_t>(P.K) +
                            C::bytes<uint8_t>(P.L) + C::bytes<float>(P.L));
        C c(h->aux_buf);
        CullArgs a;
        a.L = P.L;
        a.F = P.K;
        a.M = P.M;
        a.counters = c.take<unsigned long long>(4);
        double* Rt = c.take<double>(12 * (size_t)P.K);
        double* intr = c.take<double>(4);
        int32_t* lm_id = c.take<int32_t>(P.L);
        int32_t* frame_id = c.take<int32_t>(P.K);
        a.erase = c.take<uint8_t>(P.L);
        a.mean = c.take<float>(P.L);
        a.Rt = Rt;
        a.intr = intr;
        a.intr_stride = 0;
        a.lm = P.lm;
        a.lm_stride = kLmStride;
        a.lm_id = lm_id;
        a.obs_frame = P.obs_pose;
        a.obs_frame_id = nullptr;
        a.frame_id = frame_id;
        a.lm_gen = landmark_id_generator;
        a.frame_gen = frame_id_generator;
        const double in4[4] = {P.intr.fx, P.intr.fy, P.intr.cx, P.intr.cy};
        return cull_run(h, a, erase, mean_error, rep, [&] {
            ZS_CUDA(cudaMemcpyAsync(intr, in4, sizeof(in4), cudaMemcpyHostToDevice, h->stream));
            if (P.L > 0)
                ZS_CUDA(cudaMemcpyAsync(lm_id, landmark_id, sizeof(int32_t) * (size_t)P.L, cudaMemcpyHostToDevice,
                                        h->stream));
            if (P.K > 0)
                ZS_CUDA(cudaMemcpyAsync(frame_id, pose_frame_id, sizeof(int32_t) * (size_t)P.K,
                                        cudaMemcpyHostToDevice, h->stream));
        }, [&] {
            launch_pose_rt(P.K, P.pose, Rt, h->stream);
            launch_cull(a, P.lm_ptr, P.obs_uv, h->stream);
        });
    } catch (const CudaError& e) {
        return cuda_status(e.err);
    }
}

int zs_ba_get_history(zs_ba_handle* h, zs_ba_attempt* out, int32_t capacity, int32_t* count) {
    if (!h || !count || capacity < 0 || (capacity > 0 && !out)) return ZS_ERR_INVALID;
    const int32_t n = (int32_t)h->history.size();
    *count = n;
    for (int32_t i = 0; i < n && i < capacity; ++i) out[i] = h->history[(size_t)i];
    return ZS_OK;
}

int zs_ba_linear_step(zs_ba_handle* h, double lambda, double* S, double* bs, double* delta, double* b) {
    if (!h) return ZS_ERR_INVALID;
    if (!h->has_problem) return ZS_ERR_NO_PROBLEM;
    if (h->batch) return ZS_ERR_UNSUPPORTED;
    try {
        ZS_CUDA(cudaSetDevice(h->device));
        return h->tsize == 8 ? linear_step_impl<double>(h, lambda, S, bs, delta, b)
                             : linear_step_impl<float>(h, lambda, S, bs, delta, b);
    } catch (const CudaError& e) {
        return cuda_status(e.err);
    }
}

int zs_ba_adjoint(zs_ba_handle* h, const double* dloss_dpose, const double* dloss_dlandmark, double* dloss_duv,
                  double* dloss_dintrinsics, double* adjoint_state, zs_ba_adjoint_report* rep) {
    if (!h) return ZS_ERR_INVALID;
    if (rep) std::memset(rep, 0, sizeof(*rep));
    if (!h->has_problem) return ZS_ERR_NO_PROBLEM;
    if (h->tsize != 8 || h->P.loss.kind != ZS_LOSS_NONE || h->batch) return ZS_ERR_UNSUPPORTED;
    DevProblem& P = h->P;
    DevWork& W = h->W;
    cudaStream_t s = h->stream;
    const int n = P.n;
    const int64_t N = (int64_t)n + 3LL * P.L;
    int status = ZS_OK;
    try {
        ZS_CUDA(cudaSetDevice(h->device));
        ZS_CUDA(cudaEventRecord(h->ev0, s));
        if (!h->adj_rec) {
            h->adj_rec = dalloc<double>((size_t)std::max<int64_t>(P.M, 1) * kAdjRecord, h->owned);
            h->adj_part = dalloc<double>((size_t)std::max<int64_t>(P.M, 1) * 9, h->owned);
            h->adj_vec = dalloc<double>((size_t)std::max<int64_t>(N, 1) * 7, h->owned);
            if (n > 0 && n <= kAdjInvMaxN) h->adj_inv = dalloc<double>((size_t)n * (2 * (size_t)n + 1), h->owned);
        }
        double* a = h->adj_vec;
        double* v = a + N;
        double* r = v + N;
        double* z = r + N;
        double* pv = z + N;
        double* q = pv + N;
        double* zero = q + N;
        // a = dL/dx (local coordinates)
        std::vector<double> ah((size_t)N, 0.0);
        for (int k = 0; k < P.K && dloss_dpose; ++k)
            for (int i = 0; i < 6; ++i) ah[6 * (size_t)k + i] = dloss_dpose[6 * (size_t)k + i];
        for (int l = 0; l < P.L && dloss_dlandmark; ++l)
            for (int i = 0; i < 3; ++i) ah[(size_t)n + 3 * (size_t)l + i] = dloss_dlandmark[3 * (size_t)l + i];
        if (N > 0) ZS_CUDA(cudaMemcpyAsync(a, ah.data(), N * sizeof(double), cudaMemcpyHostToDevice, s));
        ZS_CUDA(cudaMemsetAsync(v, 0, std::max<int64_t>(N, 1) * sizeof(double), s));
        ZS_CUDA(cudaMemsetAsync(zero, 0, std::max<int64_t>(N, 1) * sizeof(double), s));
        // Gauss-Newton linearisation and its lightly damped factorisation:
        // the preconditioner M = H_GN + lambda I.
        linearize<double>(h);
        launch_adj_prep(P, h->adj_rec, s);
        launch_cost(P, W, h->st, false, s);
        launch_init_lambda(P, W, h->st, h->opt.tau, h->opt.diagonal_clamp, s);
        read_state(h);
        LmState init{};
        init.lambda = 1e-9 * std::max(h->st_host->max_diag, 1e-300);
        init.nu = 2.0;
        init.solve_ok = 1;
        ZS_CUDA(cudaMemcpyAsync(h->st, &init, sizeof(LmState), cudaMemcpyHostToDevice, s));
        launch_invert_w<double>(P, W, h->st, s);
        launch_schur<double>(P, W, h->st, s);
        ZS_CUDA((launch_factor<double, double>(n, W.S, (double*)W.F, (double*)W.D, h->st, s)));
        read_state(h);
        if (!h->st_host->solve_ok) {
            status = ZS_ERR_CHOLESKY;
        } else {
            std::vector<double> red(kReduceBlocks * 4);
            auto dot = [&](const double* x, const double* y) {
                launch_adj_dot(N, x, y, W.red, s);
                ZS_CUDA(cudaMemcpyAsync(red.data(), W.red, kReduceBlocks * sizeof(double), cudaMemcpyDeviceToHost, s));
                ZS_CUDA(cudaStreamSynchronize(s));
                double t = 0.0;
                for (int i = 0; i < kReduceBlocks; ++i) t += red[i];
                return t;
            };
            // z = M^-1 x through the Schur complement and the reduced factor;
            // up to kAdjInvMaxN the factor's inverse is formed once and each
            // reduced solve is two triangular products
            double* Xi = h->adj_inv;
            double* XiT = Xi ? Xi + (size_t)n * n : nullptr;
            if (Xi) launch_adj_tri_inverse(n, (const double*)W.F, Xi, XiT, s);
            auto precondition = [&](const double* x, double* out) {
                launch_adj_copy(N, x, W.b, s);
                launch_bs<double>(P, W, s);
                if (Xi) {
                    launch_adj_apply_inverse(n, Xi, XiT, W.bs, XiT + (size_t)n * n, W.delta, s);
                } else {
                    ZS_CUDA((launch_solve_refine<double, double>(n, W.S, (const double*)W.F, (const double*)W.D,
                                                                 W.bs, W.delta, W.work, h->st, 0, 0.0, s)));
                }
                launch_backsub<double>(P, W, h->st, s);
                launch_adj_copy(N, W.delta, out, s);
            };
            launch_adj_residual(P, h->adj_rec, v, a, h->adj_part, W.opch_sum, r, s);  // r = a, fixed entries zeroed
            const double anorm = std::sqrt(dot(r, r));
            double rn = anorm;
            int it = 0;
            const int max_it = 200;
            if (anorm > 0.0) {
                precondition(r, z);
                launch_adj_copy(N, z, pv, s);
                double rz = dot(r, z);
                if (h->opt.verbose)
                    std::fprintf(stderr, "zs adjoint: |a| %.6e  r.Mr %.6e  |M^-1 a| %.6e\n", anorm, rz,
                                 std::sqrt(dot(z, z)));
                // The iterations run with their scalars on the device
                // (AdjCg): the host enqueues kAdjBatch of them at a time and
                // reads the stop flag once per batch; iterations enqueued past
                // the stop change nothing.
                AdjCg c0{};
                c0.rz = rz;
                c0.anorm = anorm;
                c0.tol = 1e-13;
                c0.max_it = max_it;
                AdjCg* cg = reinterpret_cast<AdjCg*>(W.red + kReduceBlocks * 4);
                ZS_CUDA(cudaMemcpyAsync(cg, &c0, sizeof(AdjCg), cudaMemcpyHostToDevice, s));
                double* red2 = W.red + kReduceBlocks;  // the loop's partial sums
                AdjCg ch = c0;
                constexpr int kAdjBatch = 8;
                while (!ch.done) {
                    for (int b = 0; b < kAdjBatch; ++b) {
                        launch_adj_residual(P, h->adj_rec, pv, zero, h->adj_part, W.opch_sum, q, s);  // q = -H p
                        launch_adj_dot(N, pv, q, red2, s);
                        launch_adj_cg_pap(red2, cg, s);                // alpha = rz / p.Hp
                        launch_adj_cg_axpby(N, cg, 0, pv, v, s);       // v += alpha p
                        launch_adj_cg_axpby(N, cg, 0, q, r, s);        // r -= alpha H p
                        launch_adj_dot(N, r, r, red2, s);
                        launch_adj_cg_rn(red2, cg, s);                 // |r|, stop test
                        precondition(r, z);
                        launch_adj_dot(N, r, z, red2, s);
                        launch_adj_cg_rz(red2, cg, s);                 // beta, rz
                        launch_adj_cg_axpby(N, cg, 1, z, pv, s);       // p = z + beta p
                    }
                    ZS_CUDA(cudaMemcpyAsync(&ch, cg, sizeof(AdjCg), cudaMemcpyDeviceToHost, s));
                    ZS_CUDA(cudaStreamSynchronize(s));
                    if (h->opt.verbose)
                        std::fprintf(stderr, "zs adjoint: it %3d  |r|/|a| %.6e  done %d\n", ch.it, ch.rn / anorm,
                                     ch.done);
                }
                it = ch.it;
                // the true residual of the returned v
                launch_adj_residual(P, h->adj_rec, v, a, h->adj_part, W.opch_sum, r, s);
                rn = std::sqrt(dot(r, r));
            }
            // outputs from v
            double* duv_dev = h->adj_part;  // 2M doubles of scratch
            launch_adj_out(P, h->adj_rec, v, duv_dev, W.red, s);
            std::vector<double> duv((size_t)std::max<int64_t>(P.M, 1) * 2);
            if (P.M > 0)
                ZS_CUDA(cudaMemcpyAsync(duv.data(), duv_dev, 2 * P.M * sizeof(double), cudaMemcpyDeviceToHost, s));
            ZS_CUDA(cudaMemcpyAsync(red.data(), W.red, kReduceBlocks * 4 * sizeof(double), cudaMemcpyDeviceToHost, s));
            ZS_CUDA(cudaStreamSynchronize(s));
            if (dloss_duv)
                for (int64_t i = 0; i < P.M; ++i) {
                    dloss_duv[2 * h->perm[i]] = duv[2 * i];
                    dloss_duv[2 * h->perm[i] + 1] = duv[2 * i + 1];
                }
            if (dloss_dintrinsics)
                for (int c = 0; c < 4; ++c) {
                    double t = 0.0;
                    for (int b = 0; b < kReduceBlocks; ++b) t += red[4 * b + c];
                    dloss_dintrinsics[c] = t;
                }
            if (adjoint_state && N > 0)
                ZS_CUDA(cudaMemcpy(adjoint_state, v, N * sizeof(double), cudaMemcpyDeviceToHost));
            if (rep) {
                rep->iterations = it;
                rep->rel_residual = anorm > 0 ? rn / anorm : 0.0;
            }
        }
        ZS_CUDA(cudaEventRecord(h->ev1, s));
        ZS_CUDA(cudaEventSynchronize(h->ev1));
        float ms = 0.f;
        cudaEventElapsedTime(&ms, h->ev0, h->ev1);
        if (rep) {
            rep->ms_total = ms;
            rep->status = status;
        }
    } catch (const CudaError& e) {
        status = cuda_status(e.err);
        if (rep) rep->status = status;
    }
    return status;
}

int zs_dense_cholesky_solve(const double* A, int n, const double* b, double* Lout, double* x, int precision) {
    if (!A || n <= 0 || !b) return ZS_ERR_INVALID;
    if (precision != ZS_PRECISION_FP64 && precision != ZS_PRECISION_MIXED) return ZS_ERR_INVALID;
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count <= 0) {
        cudaGetLastError();
        return ZS_ERR_CUDA;
    }
    std::vector<void*> owned;
    cudaStream_t s = nullptr;
    int status = ZS_OK;
    try {
        ZS_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
        const size_t nn = (size_t)n * n;
        double* dA = dalloc<double>(nn, owned);
        double* db = dalloc<double>(n, owned);
        double* dx = dalloc<double>(n, owned);
        double* dwork = dalloc<double>(4 * (size_t)n + 256, owned);
        LmState* st = dalloc<LmState>(1, owned);
        LmState init{};
        init.solve_ok = 1;
        ZS_CUDA(cudaMemcpyAsync(st, &init, sizeof(init), cudaMemcpyHostToDevice, s));
        ZS_CUDA(cudaMemcpyAsync(dA, A, nn * sizeof(double), cudaMemcpyHostToDevice, s));
        ZS_CUDA(cudaMemcpyAsync(db, b, n * sizeof(double), cudaMemcpyHostToDevice, s));
        std::vector<double> Lh;
        if (precision == ZS_PRECISION_FP64) {
            double* dF = dalloc<double>(nn, owned);
            double* dD = dalloc<double>(1024 * (size_t)((n + 31) / 32), owned);
            ZS_CUDA((launch_reduced_solve<double, double>(n, dA, dF, dD, db, dx, dwork, st, 0, 0.0, s)));
            if (Lout) {
                Lh.resize(nn);
                ZS_CUDA(cudaMemcpyAsync(Lh.data(), dF, nn * sizeof(double), cudaMemcpyDeviceToHost, s));
            }
        } else {
            float* dF = dalloc<float>(nn, owned);
            float* dX = dalloc<float>(nn, owned);
            float* dXT = dalloc<float>(nn, owned);
            int* flags = dalloc<int>((size_t)dag_flag_ints(n), owned);
            int epoch = 0;
            ZS_CUDA(cudaMemsetAsync(flags, 0, sizeof(int) * (size_t)dag_flag_ints(n), s));
            // the factor as the mixed solve forms it, without the shifted retry
            // (st->skip_factor stays 0, so the solve test applies)
            float* scratch = chol_tc_applies(n) ? dalloc<float>((size_t)chol_tc_scratch_floats(n), owned) : nullptr;
            TcStreams tcs;
            if (scratch) ZS_CUDA(tcs.init(n));
            ZS_CUDA((launch_factor_dag(n, dA, dF, dX, dXT, scratch, scratch ? &tcs : nullptr, st, flags, &epoch, s)));
            ZS_CUDA((launch_refine<double, float>(n, dA, dX, dXT, db, dx, dwork, st, 10, 1e-14, s)));
            if (Lout) {
                std::vector<float> tmp(nn);
                ZS_CUDA(cudaMemcpyAsync(tmp.data(), dF, nn * sizeof(float), cudaMemcpyDeviceToHost, s));
                ZS_CUDA(cudaStreamSynchronize(s));
                Lh.assign(tmp.begin(), tmp.end());
            }
        }
        LmState out{};
        ZS_CUDA(cudaMemcpyAsync(&out, st, sizeof(out), cudaMemcpyDeviceToHost, s));
        if (x) ZS_CUDA(cudaMemcpyAsync(x, dx, n * sizeof(double), cudaMemcpyDeviceToHost, s));
        ZS_CUDA(cudaStreamSynchronize(s));
        ZS_CUDA(cudaGetLastError());
        if (Lout) {
            for (int i = 0; i < n; ++i)
                for (int j = 0; j < n; ++j) Lout[(size_t)i * n + j] = (j <= i) ? Lh[(size_t)i * n + j] : 0.0;
        }
        status = out.timeout ? ZS_ERR_TIMEOUT : (out.solve_ok ? ZS_OK : ZS_ERR_CHOLESKY);
    } catch (const CudaError& e) {
        status = cuda_status(e.err);
    }
    if (s) cudaStreamSynchronize(s);
    for (void* p : owned) cudaFree(p);
    if (s) cudaStreamDestroy(s);
    return status;
}

}  // extern "C"

// ------------------------------------------------------------ batched windows

namespace {

// Version of the window-solve kernel the tuning results belong to.
constexpr const char* kTuneKernel = "bsolve-tiles32-v2";

// Autotuned reduced-solve block sizes per (device name, precision, bucket),
// shared by all handles of the process and optionally kept in a file:
// one JSON object per line inside {"entries": [ ... ]}.
struct TuneCache {
    std::mutex mu;
    std::map<std::tuple<std::string, int, int>, int> threads;
    std::set<std::string> loaded;
};

TuneCache& tune_cache() {
    static TuneCache c;
    return c;
}

// Returns false when a path is given but no cache file exists there yet.
bool tune_load_locked(TuneCache& c, const char* path) {
    if (!path) return true;
    FILE* f = std::fopen(path, "r");
    if (!f) return false;
    if (c.loaded.count(path)) {
        std::fclose(f);
        return true;
    }
    c.loaded.insert(path);
    char line[512];
    while (std::fgets(line, sizeof(line), f)) {
        char dev[256] = {0}, prec[16] = {0};
        int bucket = -1, threads = 0;
        char kern[64] = {0};
        if (std::sscanf(line, " {\"kernel\": \"%63[^\"]\", \"device\": \"%255[^\"]\", \"precision\": \"%15[^\"]\", "
                              "\"bucket\": %d, \"threads\": %d",
                        kern, dev, prec, &bucket, &threads) == 5 &&
            std::strcmp(kern, kTuneKernel) == 0 &&
            bucket >= 0 && bucket < kBatchBuckets &&
            (threads == 64 || threads == 128 || threads == 256 || threads == 512 || threads == 1024)) {
            const int ts = std::strcmp(prec, "fp64") == 0 ? 8 : 4;
            c.threads[std::make_tuple(std::string(dev), ts, bucket)] = threads;
        }
    }
    std::fclose(f);
    return true;
}

void tune_save_locked(TuneCache& c, const char* path) {
    if (!path) return;
    FILE* f = std::fopen(path, "w");
    if (!f) return;
    std::fprintf(f, "{\"entries\": [\n");
    size_t i = 0;
    for (const auto& e : c.threads) {
        std::fprintf(f, "  {\"kernel\": \"%s\", \"device\": \"%s\", \"precision\": \"%s\", \"bucket\": %d, \"threads\": %d}%s\n",
                     kTuneKernel, std::get<0>(e.first).c_str(), std::get<1>(e.first) == 8 ? "fp64" : "mixed", std::get<2>(e.first),
                     e.second, ++i < c.threads.size() ? "," : "");
    }
    std::fprintf(f, "]}\n");
    std::fclose(f);
}

// Block size of each present bucket: from the cache, else timed now.
template <typename T>
void batch_tune(zs_ba_handle* h) {
    BatchDev& B = h->B;
    int sms = 0;
    ZS_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, h->device));
    cudaDeviceProp prop;
    ZS_CUDA(cudaGetDeviceProperties(&prop, h->device));
    TuneCache& c = tune_cache();
    std::lock_guard<std::mutex> lock(c.mu);
    bool tuned = !tune_load_locked(c, h->opt.autotune_cache);
    for (int b = 0; b < kBatchBuckets; ++b) {
        const int cnt = B.bucket_off[b + 1] - B.bucket_off[b];
        if (cnt == 0 || B.threads[b] > 0) continue;
        const auto key = std::make_tuple(std::string(prop.name), (int)sizeof(T), b);
        auto it = c.threads.find(key);
        int t = 0;
        if (it != c.threads.end()) {
            t = it->second;
            h->tune_us[b] = 0.f;
        } else {
            int bps = 0;
            float us = 0.f;
            ZS_CUDA(bsolve_autotune<T>(b, sms, h->stream, &t, &bps, &us));
            c.threads[key] = t;
            h->tune_us[b] = us;
            tuned = true;
        }
        const int per_sm = bsolve_max_blocks_per_sm<T>(b, t);  // also sets the kernel's shared-memory limit
        if (per_sm <= 0) throw CudaError{cudaErrorInvalidConfiguration};
        B.threads[b] = t;
        B.blocks[b] = std::min(cnt, per_sm * sms);
    }
    if (tuned) tune_save_locked(c, h->opt.autotune_cache);
}

BatchParams batch_params(const zs_ba_handle* h, int iterations, bool use_relative) {
    const zs_ba_options& o = h->opt;
    BatchParams prm{};
    prm.iterations = iterations;
    prm.use_relative = use_relative ? 1 : 0;
    prm.max_failures = o.max_failures;
    prm.refine_iters = std::max(0, o.refine_iterations);
    prm.max_rounds = std::max(1, iterations) * std::max(1, o.max_failures) + 1;
    prm.use_cond = 0;
    prm.relative_tolerance = o.relative_tolerance;
    prm.chi2_floor = o.chi2_floor;
    prm.legacy_stop = o.legacy_stop;
    prm.tau = o.tau;
    prm.clamp = o.diagonal_clamp;
    prm.refine_tol = o.refine_tolerance;
    prm.cond = 0;
    return prm;
}

// The batched solve as one graph: prologue (child graph), then a
// conditional WHILE node whose body is one attempt round; the round's last
// kernel sets the condition to "any window still active".
template <typename T>
void build_batch_graph(zs_ba_handle* h, BatchParams prm) {
    cudaStream_t s = h->stream;
    ZS_CUDA(cudaGraphCreate(&h->bgraph, 0));
    cudaGraph_t pro = nullptr;
    long long c0 = launch_counter();
    ZS_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    launch_batch_prologue<T>(h->P, h->W, h->B, prm, s);
    ZS_CUDA(cudaStreamEndCapture(s, &pro));
    h->bpro_launches = launch_counter() - c0;
    cudaGraphNode_t npro = nullptr;
    const cudaError_t ea = cudaGraphAddChildGraphNode(&npro, h->bgraph, nullptr, 0, pro);
    cudaGraphDestroy(pro);
    ZS_CUDA(ea);
    cudaGraphConditionalHandle cond = 0;
    ZS_CUDA(cudaGraphConditionalHandleCreate(&cond, h->bgraph, 1, cudaGraphCondAssignDefault));
    cudaGraphNodeParams cp = {cudaGraphNodeTypeConditional};
    cp.conditional.handle = cond;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    cudaGraphNode_t nloop = nullptr;
    ZS_CUDA(cudaGraphAddNode(&nloop, h->bgraph, &npro, nullptr, 1, &cp));
    cudaGraph_t body = cp.conditional.phGraph_out[0];
    prm.use_cond = 1;
    prm.cond = cond;
    c0 = launch_counter();
    ZS_CUDA(cudaStreamBeginCaptureToGraph(s, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
    const cudaError_t el = launch_batch_round<T>(h->P, h->W, h->B, prm, s);
    cudaGraph_t body_out = nullptr;
    const cudaError_t ee = cudaStreamEndCapture(s, &body_out);
    ZS_CUDA(el);
    ZS_CUDA(ee);
    h->bbody_launches = launch_counter() - c0;
    ZS_CUDA(cudaGraphInstantiate(&h->bexec, h->bgraph, 0));
}

template <typename T>
int solve_batch_impl(zs_ba_handle* h, int iterations, bool use_relative, zs_ba_report* wr, zs_ba_batch_report* rep) {
    const DevProblem& P = h->P;
    BatchDev& B = h->B;
    cudaStream_t s = h->stream;
    zs_ba_batch_report r{};
    r.windows = P.nwin;
    const bool po = pose_only_batch(h);
    if (!po) batch_tune<T>(h);
    for (int b = 0; b < kBatchBuckets; ++b) {
        r.bucket_windows[b] = B.bucket_off[b + 1] - B.bucket_off[b];
        r.bucket_threads[b] = B.threads[b];
        r.bucket_tune_us[b] = h->tune_us[b];
    }
    BatchParams prm = batch_params(h, iterations, use_relative);
    if (h->opt.profile && !B.prof) {
        B.prof = dalloc<long long>((size_t)P.nwin * kBatchProfSlots, h->owned);
        h->release_graph();  // the captured kernels must see the profile buffer
    }
    if (B.prof) ZS_CUDA(cudaMemsetAsync(B.prof, 0, sizeof(long long) * P.nwin * kBatchProfSlots, s));
    const long long launches0 = launch_counter();
    if (po) {
        const zs_ba_options& o = h->opt;
        PoseOnlyCtl ctl{o.tau, o.diagonal_clamp, o.legacy_stop, o.relative_tolerance, o.chi2_floor,
                        o.max_failures, iterations, use_relative ? 1 : 0, 0};
        ZS_CUDA(cudaEventRecord(h->ev0, s));
        ZS_CUDA(launch_pose_only_windows(h->P, ctl, B.ctl, B.st, s));
        ZS_CUDA(cudaEventRecord(h->ev1, s));
    } else if (h->opt.batch_graph) {
        if (!h->bexec || h->bgraph_iters != iterations || h->bgraph_rel != (int)use_relative) {
            h->release_graph();
            build_batch_graph<T>(h, prm);
            h->bgraph_iters = iterations;
            h->bgraph_rel = use_relative ? 1 : 0;
        }
        ZS_CUDA(cudaEventRecord(h->ev0, s));
        ZS_CUDA(cudaGraphLaunch(h->bexec, s));
        ZS_CUDA(cudaEventRecord(h->ev1, s));
        r.graph_launches = 1;
    } else {
        ZS_CUDA(cudaEventRecord(h->ev0, s));
        launch_batch_prologue<T>(h->P, h->W, B, prm, s);
        int any = 1;
        while (any) {
            ZS_CUDA(launch_batch_round<T>(h->P, h->W, B, prm, s));
            ZS_CUDA(cudaMemcpyAsync(&any, B.any_active, sizeof(int), cudaMemcpyDeviceToHost, s));
            ZS_CUDA(cudaStreamSynchronize(s));
        }
        ZS_CUDA(cudaEventRecord(h->ev1, s));
    }
    ZS_CUDA(cudaEventSynchronize(h->ev1));
    ZS_CUDA(cudaGetLastError());
    float ms = 0.f;
    ZS_CUDA(cudaEventElapsedTime(&ms, h->ev0, h->ev1));
    std::vector<LmState> st(P.nwin);
    std::vector<WinCtl> ctl(P.nwin);
    int rounds = 0;
    ZS_CUDA(cudaMemcpyAsync(st.data(), B.st, sizeof(LmState) * P.nwin, cudaMemcpyDeviceToHost, s));
    ZS_CUDA(cudaMemcpyAsync(ctl.data(), B.ctl, sizeof(WinCtl) * P.nwin, cudaMemcpyDeviceToHost, s));
    if (!po) ZS_CUDA(cudaMemcpyAsync(&rounds, B.rounds, sizeof(int), cudaMemcpyDeviceToHost, s));
    ZS_CUDA(cudaStreamSynchronize(s));
    if (po)  // a window's attempts run back to back in its CTA: the longest is the rounds' count
        for (const WinCtl& c : ctl) rounds = std::max(rounds, c.attempts);
    r.rounds = rounds;
    r.ms_total = ms;
    r.kernel_launches = r.graph_launches ? h->bpro_launches + (long long)rounds * h->bbody_launches
                                         : launch_counter() - launches0;
    int64_t accepted = 0;
    for (int w = 0; w < P.nwin; ++w) {
        accepted += ctl[w].accepted;
        r.attempts += ctl[w].attempts;
        if (!wr) continue;
        zs_ba_report& o = wr[w];
        std::memset(&o, 0, sizeof(o));
        o.status = ZS_OK;
        o.iterations = ctl[w].iterations;
        o.accepted = ctl[w].accepted;
        o.attempts = ctl[w].attempts;
        o.cholesky_failures = ctl[w].chol_failures;
        o.refine_sweeps = ctl[w].refine_sweeps;
        o.chi2_initial = ctl[w].chi2_initial;
        o.chi2_final = st[w].chi2;
        o.lambda_final = st[w].lambda;
        o.ms_total = ms;
    }
    r.accepted = accepted;
    r.status = ZS_OK;
    if (rep) *rep = r;
    return (int)std::min<int64_t>(accepted, 0x7fffffff);
}

}  // namespace

extern "C" {

int zs_ba_set_batch(zs_ba_handle* h, int num_windows, const zs_ba_problem* windows) {
    if (!h || !windows || num_windows <= 0 || num_windows > 65535) return ZS_ERR_INVALID;
    int64_t K = 0, L = 0, M = 0;
    for (int w = 0; w < num_windows; ++w) {
        const zs_ba_problem& p = windows[w];
        const int v = validate(&p);
        if (v != ZS_OK) return v;
        if (p.num_poses > ZS_BATCH_MAX_POSES) return ZS_ERR_UNSUPPORTED;
        if (w > 0) {
            const zs_ba_problem& q = windows[0];
            for (int i = 0; i < 4; ++i)
                if (p.intrinsics[i] != q.intrinsics[i]) return ZS_ERR_UNSUPPORTED;
            if (p.loss_kind != q.loss_kind || p.loss_delta != q.loss_delta) return ZS_ERR_UNSUPPORTED;
            if ((p.obs_info != nullptr) != (q.obs_info != nullptr)) return ZS_ERR_UNSUPPORTED;
        }
        K += p.num_poses;
        L += p.num_landmarks;
        M += p.num_obs;
    }
    if (K > 0x7fffffffLL / 6 || L > 0x7fffffffLL / 3 || M > 0x7fffffffLL) return ZS_ERR_INVALID;
    try {
        // the windows concatenated: poses, landmarks and observations in window order
        std::vector<double> poses(7 * K), lms(3 * L), uv(2 * M);
        std::vector<uint8_t> pf(K), lf(L);
        std::vector<int32_t> op(M), ol(M);
        const bool has_info = windows[0].obs_info != nullptr;
        std::vector<double> info(has_info ? 4 * M : 0);
        std::vector<int32_t> wp{0}, wl{0};
        int64_t k0 = 0, l0 = 0, o0 = 0;
        for (int w = 0; w < num_windows; ++w) {
            const zs_ba_problem& p = windows[w];
            if (p.num_poses) {
                std::memcpy(&poses[7 * k0], p.poses, sizeof(double) * 7 * p.num_poses);
                std::memcpy(&pf[k0], p.pose_fixed, p.num_poses);
            }
            if (p.num_landmarks) {
                std::memcpy(&lms[3 * l0], p.landmarks, sizeof(double) * 3 * p.num_landmarks);
                std::memcpy(&lf[l0], p.landmark_fixed, p.num_landmarks);
            }
            for (int64_t o = 0; o < p.num_obs; ++o) {
                op[o0 + o] = (int32_t)(k0 + p.obs_pose[o]);
                ol[o0 + o] = (int32_t)(l0 + p.obs_landmark[o]);
                uv[2 * (o0 + o)] = p.obs_uv[2 * o];
                uv[2 * (o0 + o) + 1] = p.obs_uv[2 * o + 1];
                if (has_info)
                    for (int i = 0; i < 4; ++i) info[4 * (o0 + o) + i] = p.obs_info[4 * o + i];
            }
            k0 += p.num_poses;
            l0 += p.num_landmarks;
            o0 += p.num_obs;
            wp.push_back((int32_t)k0);
            wl.push_back((int32_t)l0);
        }
        zs_ba_problem cat = windows[0];
        cat.num_poses = (int32_t)K;
        cat.num_landmarks = (int32_t)L;
        cat.num_obs = M;
        cat.poses = poses.data();
        cat.pose_fixed = pf.data();
        cat.landmarks = lms.data();
        cat.landmark_fixed = lf.data();
        cat.obs_pose = op.data();
        cat.obs_landmark = ol.data();
        cat.obs_uv = uv.data();
        cat.obs_info = has_info ? info.data() : nullptr;

        ZS_CUDA(cudaSetDevice(h->device));
        ZS_CUDA(cudaStreamSynchronize(h->stream));
        h->release_problem(true);
        build_problem(h, &cat, &wp, &wl);
        // windows by reduced-system size bucket, largest first within a bucket
        BatchDev& B = h->B;
        std::vector<std::vector<int32_t>> byb(kBatchBuckets);
        for (int w = 0; w < num_windows; ++w) byb[batch_bucket(6 * (wp[w + 1] - wp[w]))].push_back(w);
        std::vector<int32_t> lists;
        B.bucket_off[0] = 0;
        for (int b = 0; b < kBatchBuckets; ++b) {
            std::stable_sort(byb[b].begin(), byb[b].end(),
                             [&](int32_t a, int32_t c) { return wp[a + 1] - wp[a] > wp[c + 1] - wp[c]; });
            lists.insert(lists.end(), byb[b].begin(), byb[b].end());
            B.bucket_off[b + 1] = (int)lists.size();
        }
        auto& own = h->owned;
        ZS_CUDA(cudaEventCreateWithFlags(&B.ev_fork, cudaEventDisableTiming));
        for (int b = 0; b < kBatchBuckets; ++b) {
            ZS_CUDA(cudaStreamCreateWithFlags(&B.streams[b], cudaStreamNonBlocking));
            ZS_CUDA(cudaEventCreateWithFlags(&B.ev_join[b], cudaEventDisableTiming));
        }
        B.lists = upload(lists, own, h->stream);
        B.st = dalloc<LmState>(num_windows, own);
        B.ctl = dalloc<WinCtl>(num_windows, own);
        B.counters = dalloc<int>(kBatchBuckets, own);
        B.any_active = dalloc<int>(1, own);
        B.rounds = dalloc<int>(1, own);
        ZS_CUDA(cudaMemsetAsync(B.st, 0, sizeof(LmState) * num_windows, h->stream));
        ZS_CUDA(cudaMemsetAsync(B.ctl, 0, sizeof(WinCtl) * num_windows, h->stream));
        ZS_CUDA(cudaMemsetAsync(B.rounds, 0, sizeof(int), h->stream));
        ZS_CUDA(cudaStreamSynchronize(h->stream));
        h->owned.trim();
        h->wpose0 = wp;
        h->wlm0 = wl;
        h->batch = true;
        h->has_problem = true;
    } catch (const CudaError& e) {
        h->release_problem();
        return cuda_status(e.err);
    } catch (const std::bad_alloc&) {
        h->release_problem();
        return ZS_ERR_OUT_OF_MEMORY;
    }
    return ZS_OK;
}

int zs_ba_solve_batch(zs_ba_handle* h, int iterations, int use_relative, zs_ba_report* window_reports,
                      zs_ba_batch_report* rep) {
    if (!h) return ZS_ERR_INVALID;
    if (rep) std::memset(rep, 0, sizeof(*rep));
    if (!h->has_problem) return ZS_ERR_NO_PROBLEM;
    if (!h->batch) return ZS_ERR_INVALID;
    if (mixed_tukey(h) && !pose_only_batch(h)) return ZS_ERR_UNSUPPORTED;
    if (iterations < 0) return ZS_ERR_INVALID;
    try {
        ZS_CUDA(cudaSetDevice(h->device));
        return h->tsize == 8 ? solve_batch_impl<double>(h, iterations, use_relative != 0, window_reports, rep)
                             : solve_batch_impl<float>(h, iterations, use_relative != 0, window_reports, rep);
    } catch (const CudaError& e) {
        const int st = cuda_status(e.err);
        if (rep) rep->status = st;
        return st;
    }
}

int zs_ba_batch_solve_profile(zs_ba_handle* h, long long* out) {
    if (!h || !out) return ZS_ERR_INVALID;
    if (!h->has_problem) return ZS_ERR_NO_PROBLEM;
    if (!h->batch || !h->B.prof) return ZS_ERR_INVALID;
    try {
        ZS_CUDA(cudaSetDevice(h->device));
        ZS_CUDA(cudaMemcpyAsync(out, h->B.prof, sizeof(long long) * h->P.nwin * kBatchProfSlots,
                                cudaMemcpyDeviceToHost, h->stream));
        ZS_CUDA(cudaStreamSynchronize(h->stream));
    } catch (const CudaError& e) {
        return cuda_status(e.err);
    }
    return ZS_OK;
}

int zs_ba_get_window_state(zs_ba_handle* h, int window, double* poses, double* landmarks) {
    if (!h) return ZS_ERR_INVALID;
    if (!h->has_problem) return ZS_ERR_NO_PROBLEM;
    if (!h->batch || window < 0 || window >= h->P.nwin) return ZS_ERR_INVALID;
    const DevProblem& P = h->P;
    const int k0 = h->wpose0[window], nk = h->wpose0[window + 1] - k0;
    const int l0 = h->wlm0[window], nl = h->wlm0[window + 1] - l0;
    try {
        ZS_CUDA(cudaSetDevice(h->device));
        if (poses && nk > 0) {
            ZS_CUDA(cudaMemcpy2DAsync(poses, 7 * sizeof(double), P.pose + (size_t)k0 * kPoseStride,
                                      kPoseStride * sizeof(double), 7 * sizeof(double), nk, cudaMemcpyDeviceToHost,
                                      h->stream));
        }
        if (landmarks && nl > 0) {
            ZS_CUDA(cudaMemcpy2DAsync(landmarks, 3 * sizeof(double), P.lm + (size_t)l0 * kLmStride,
                                      kLmStride * sizeof(double), 3 * sizeof(double), nl, cudaMemcpyDeviceToHost,
                                      h->stream));
        }
        ZS_CUDA(cudaStreamSynchronize(h->stream));
    } catch (const CudaError& e) {
        return cuda_status(e.err);
    }
    return ZS_OK;
}

}  // extern "C"
