// Cahn-Hilliard serving: a request loop with continuous batching over resident simulations.
//
// Requests (grid size n, step count, initial field, arrival time) arrive over time. The loop admits
// arrived requests first-come first-served while their device memory fits the HBM budget: their two
// field buffers, work field, h field and row ends are allocated stream-ordered (cudaMallocAsync, no device
// synchronisation) and their pre-factored solver table is shared by every resident grid of the same
// size. All resident grids then advance together, a chunk of steps at a time, through the same
// persistent kernels as the batch solver (ch_solver.cu): one launch per kernel covers every grid.
// Between chunks, finished grids are read back and their memory is released, and new arrivals join,
// so work that arrives while others are on the GPU overlaps with them. Each grid is computed by the
// same operations whatever else is resident, so a result is bit-identical alone and in the mix.
//
// The solver is the reference's (cuPentCahnADI/src/cuPentCahnADI.cu:197-627); the request loop has
// no counterpart in the reference, whose driver runs one simulation per process.
#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>   // header-only; the ranges cost nothing unless a profiler is attached

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <thread>
#include <vector>

#include "../../include/custen_gb300.h"
#include "ch_internal.cuh"

namespace custen {
namespace ch {

// Counter-based uniform initial field U(lo, hi) from a seed (splitmix64 of seed and index).
__global__ void ch_fill_uniform_kernel(double* f, long long count, unsigned long long seed, double lo, double hi) {
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < count;
         k += (long long)gridDim.x * blockDim.x) {
        unsigned long long z = seed * 0x9E3779B97F4A7C15ull + (unsigned long long)k + 1ull;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        z ^= z >> 31;
        const double u = (double)(z >> 11) * (1.0 / 9007199254740992.0);   // [0, 1)
        f[k] = lo + u * (hi - lo);
    }
}

struct Request {
    int n = 0;
    double lx = 0.0;
    int steps = 0;
    double arrival = 0.0;            // seconds on the server clock
    std::vector<double> c0;          // host initial field (empty: generated on the device from seed)
    unsigned long long seed = 0;
    int state = 0;                   // 0 pending, 1 resident, 2 done, 3 failed (see error)
    int inject = 0;                  // test hook: 1 = the device allocation at admission fails
    std::string error;
    std::vector<double> c_old0;      // host cOld to resume from (empty: cOld = c0, a fresh start)
    double time = 0.0;               // simulated time, advanced by dt per step as the reference does
    int done_steps = 0;
    int snap_every = 0;              // write a snapshot every snap_every steps (0: none)
    std::string snap_dir;
    int snaps = 0;
    int remaining = 0;
    double admit_t = -1.0, done_t = -1.0;
    double mean0 = 0.0, mean_end = 0.0;
    std::vector<double> result;
    size_t bytes = 0;
    GridDev g{};
    std::string table_key;
};

struct TableRef {
    double* ptr = nullptr;
    int refs = 0;
    size_t bytes = 0;
};

struct Server {
    int device = 0;
    cudaStream_t stream = nullptr;
    int rhs_fp32 = 0;
    double gamma = 0.01, dt_factor = 0.1;
    double budget = 0.0;
    double used = 0.0;
    int chunk = 8;
    int keep_results = 1;
    int parity = 0;
    std::vector<Request> reqs;
    std::vector<int> active;        // request ids resident on the device
    std::map<std::string, TableRef> tables;
    GridDev* grids_d = nullptr;
    Item* items_rhs_d = nullptr;
    Item* items_rows_d = nullptr;
    size_t cap_grids = 0, cap_rhs = 0, cap_rows = 0;
    int n_rhs = 0, n_rows = 0;
    unsigned int* counters = nullptr;
    double* mass_d = nullptr;
    int sms = 0;
    // statistics of the last run
    double makespan = 0.0;
    long long total_steps = 0;
    double total_pt_steps = 0.0;
    int max_active = 0;
    double max_used = 0.0;
    unsigned long long launches = 0;
    int failed = 0;
};

static thread_local std::string g_srv_err;
static int srv_fail(cudaError_t e, const char* what) {
    g_srv_err = std::string("Error while '") + what + "': " + cudaGetErrorString(e);
    cudaGetLastError();
    return 1;
}
static int srv_arg(const std::string& m) {
    g_srv_err = m;
    return 2;
}
#define SRV_TRY(x, what)                                \
    do {                                                \
        cudaError_t _e = (x);                           \
        if (_e != cudaSuccess) return srv_fail(_e, what); \
    } while (0)

// per grid: cCurr, cOld, the work field and the h field of the two-pass right-hand side, plus 2 n row ends
static size_t grid_bytes(int n) { return 4 * (size_t)n * n * sizeof(double) + 2 * (size_t)n * sizeof(double); }

static int grow(void** p, size_t* cap, size_t need, size_t elem, cudaStream_t s) {
    if (need <= *cap) return 0;
    size_t nc = std::max(need, *cap * 2 + 16);
    if (*p) SRV_TRY(cudaFreeAsync(*p, s), "Releasing a work list");
    SRV_TRY(cudaMallocAsync(p, nc * elem, s), "Allocating a work list");
    *cap = nc;
    return 0;
}

// Rebuild the device work lists of the resident grids (largest first).
static int rebuild(Server* S) {
    std::vector<int> order = S->active;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return S->reqs[a].n > S->reqs[b].n; });
    std::vector<GridDev> grids;
    std::vector<Item> rhs, rows;
    for (size_t k = 0; k < order.size(); ++k) {
        const Request& r = S->reqs[order[k]];
        grids.push_back(r.g);
        const int bpr = r.n / BLK;
        for (int b = 0; b < bpr * bpr; ++b) rhs.push_back({(int)k, b});
        for (int b = 0; b < bpr; ++b) rows.push_back({(int)k, b});
    }
    int st;
    if ((st = grow((void**)&S->grids_d, &S->cap_grids, grids.size(), sizeof(GridDev), S->stream))) return st;
    if ((st = grow((void**)&S->items_rhs_d, &S->cap_rhs, rhs.size(), sizeof(Item), S->stream))) return st;
    if ((st = grow((void**)&S->items_rows_d, &S->cap_rows, rows.size(), sizeof(Item), S->stream))) return st;
    // pageable copies: the host vectors may be released as soon as the calls return
    SRV_TRY(cudaMemcpyAsync(S->grids_d, grids.data(), grids.size() * sizeof(GridDev), cudaMemcpyHostToDevice,
                            S->stream), "Uploading grid descriptors");
    SRV_TRY(cudaMemcpyAsync(S->items_rhs_d, rhs.data(), rhs.size() * sizeof(Item), cudaMemcpyHostToDevice, S->stream),
            "Uploading work list");
    SRV_TRY(cudaMemcpyAsync(S->items_rows_d, rows.data(), rows.size() * sizeof(Item), cudaMemcpyHostToDevice,
                            S->stream), "Uploading work list");
    S->n_rhs = (int)rhs.size();
    S->n_rows = (int)rows.size();
    return 0;
}

// Admission of one request. Returns 0 when it is resident, kAdmitFailed when it failed on its own
// (an allocation or upload error: its partial allocations are released, the error is recorded in the
// request, and the server keeps serving the others), or a fatal status when the device context itself
// reports an error.
constexpr int kAdmitFailed = -1;

static int admit(Server* S, int id, double now) {
    Request& r = S->reqs[id];
    nvtxRangePushA("admit");
    char key[128];
    snprintf(key, sizeof(key), "%d/%.17g", r.n, r.lx);
    r.table_key = key;
    TableRef& t = S->tables[key];
    cudaError_t e = cudaSuccess;
    const char* what = "";
    auto step = [&](cudaError_t x, const char* w) {
        if (e == cudaSuccess && x != cudaSuccess) {
            e = x;
            what = w;
        }
    };
    // a fake of the failing allocation call, for tests of failure isolation: nothing is allocated
    auto alloc = [&](double** p, size_t bytes) {
        return r.inject == 1 ? cudaErrorMemoryAllocation : cudaMallocAsync(p, bytes, S->stream);
    };
    bool new_table = false;
    if (!t.ptr) {
        std::vector<double> h = build_table(r.n, r.lx, S->gamma, S->dt_factor);
        t.bytes = h.size() * sizeof(double);
        step(alloc(&t.ptr, t.bytes), "Allocating a solver table");
        if (e == cudaSuccess) {
            new_table = true;
            // pageable source: the call returns once the vector has been read
            step(cudaMemcpyAsync(t.ptr, h.data(), t.bytes, cudaMemcpyHostToDevice, S->stream), "Uploading a table");
        }
    }
    const size_t f = (size_t)r.n * r.n * sizeof(double);
    double* p[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};   // cCurr, cOld, tmp, row ends, h
    for (int k = 0; k < 5 && e == cudaSuccess; ++k)
        step(alloc(&p[k], k == 3 ? 2 * (size_t)r.n * sizeof(double) : f), "Allocating a grid");
    double m = 0.0;
    if (e == cudaSuccess) {
        if (!r.c0.empty()) {
            step(cudaMemcpyAsync(p[0], r.c0.data(), f, cudaMemcpyHostToDevice, S->stream), "Uploading c0");
        } else {
            const long long count = (long long)r.n * r.n;
            ch_fill_uniform_kernel<<<std::min<long long>((count + 255) / 256, 4096), 256, 0, S->stream>>>(
                p[0], count, r.seed, -0.1, 0.1);
            step(cudaGetLastError(), "Generating c0");
        }
        if (!r.c_old0.empty())
            step(cudaMemcpyAsync(p[1], r.c_old0.data(), f, cudaMemcpyHostToDevice, S->stream), "Uploading cOld");
        else
            step(cudaMemcpyAsync(p[1], p[0], f, cudaMemcpyDeviceToDevice, S->stream), "Copying c0");
        if (e == cudaSuccess) ch_mass_kernel<<<1, 256, 0, S->stream>>>(p[0], (long long)r.n * r.n, S->mass_d);
        step(cudaMemcpyAsync(&m, S->mass_d, sizeof(double), cudaMemcpyDeviceToHost, S->stream), "Reading mass");
        step(cudaStreamSynchronize(S->stream), "Admitting");
    }
    if (e != cudaSuccess) {
        cudaGetLastError();   // clear a non-sticky error (an allocation failure is one)
        for (double* q : p)
            if (q) cudaFreeAsync(q, S->stream);
        if (new_table) {
            cudaFreeAsync(t.ptr, S->stream);
            t.ptr = nullptr;
        }
        r.state = 3;
        r.error = std::string("Error while '") + what + "': " + cudaGetErrorString(e);
        r.done_t = now;
        ++S->failed;
        nvtxRangePop();
        // a sticky error (the context is lost) ends the run; anything else stays with this request
        const cudaError_t ctx = cudaStreamSynchronize(S->stream);
        if (ctx != cudaSuccess) return srv_fail(ctx, "Admitting (device context lost)");
        return kAdmitFailed;
    }
    if (new_table) S->used += (double)t.bytes;
    ++t.refs;
    r.g.buf[S->parity] = p[0];        // cCurr
    r.g.buf[S->parity ^ 1] = p[1];    // cOld
    r.g.tmp = p[2];
    r.g.ends = p[3];
    r.g.hbuf = p[4];
    r.g.tab = t.ptr;
    r.g.n = r.n;
    r.mean0 = m / ((double)r.n * r.n);
    r.bytes = grid_bytes(r.n);
    S->used += (double)r.bytes;
    r.state = 1;
    r.remaining = r.steps;
    r.admit_t = now;
    S->active.push_back(id);
    nvtxRangePop();
    return 0;
}

static int retire(Server* S, int id, double now_after) {
    Request& r = S->reqs[id];
    const double* cur = r.g.buf[S->parity];
    ch_mass_kernel<<<1, 256, 0, S->stream>>>(cur, (long long)r.n * r.n, S->mass_d);
    double m = 0.0;
    SRV_TRY(cudaMemcpyAsync(&m, S->mass_d, sizeof(double), cudaMemcpyDeviceToHost, S->stream), "Reading mass");
    if (S->keep_results) {
        r.result.resize((size_t)r.n * r.n);
        SRV_TRY(cudaMemcpyAsync(r.result.data(), cur, r.result.size() * sizeof(double), cudaMemcpyDeviceToHost,
                                S->stream), "Reading a result");
    }
    SRV_TRY(cudaStreamSynchronize(S->stream), "Retiring");
    r.mean_end = m / ((double)r.n * r.n);
    r.done_t = now_after;
    for (double* p : {r.g.buf[0], r.g.buf[1], r.g.tmp, r.g.ends, r.g.hbuf}) SRV_TRY(cudaFreeAsync(p, S->stream), "Freeing a grid");
    S->used -= (double)r.bytes;
    TableRef& t = S->tables[r.table_key];
    if (--t.refs == 0) {
        SRV_TRY(cudaFreeAsync(t.ptr, S->stream), "Freeing a table");
        S->used -= (double)t.bytes;
        t.ptr = nullptr;
    }
    r.state = 2;
    return 0;
}

// Snapshot of a resident request after its done_steps-th step: the reference's Print_Out file
// (cuPentCahnADI.cu:103-140, name cahn_hilliard_<time %0.10lf>.nc, dataset "c") with "c_old" and "t"
// added so that the request can be resumed (custen_ch_server_submit_snapshot). Returns false with
// *err set when reading back or writing fails.
static bool write_snapshot(Server* S, Request& r, std::string* err) {
    const size_t count = (size_t)r.n * r.n;
    std::vector<double> cur(count), old(count);
    cudaError_t e = cudaMemcpyAsync(cur.data(), r.g.buf[S->parity], count * sizeof(double), cudaMemcpyDeviceToHost,
                                    S->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(old.data(), r.g.buf[S->parity ^ 1], count * sizeof(double), cudaMemcpyDeviceToHost,
                            S->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(S->stream);
    if (e != cudaSuccess) {
        *err = std::string("Error while 'Reading a snapshot': ") + cudaGetErrorString(e);
        return false;
    }
    char num[64];
    snprintf(num, sizeof(num), "%0.10f", r.time);
    const std::string path = r.snap_dir + "/cahn_hilliard_" + num + ".nc";
    const char* names[3] = {"c", "c_old", "t"};
    const double* data[3] = {cur.data(), old.data(), &r.time};
    const long long dims[6] = {r.n, r.n, r.n, r.n, 1, 1};
    if (custen_h5_write(path.c_str(), 3, names, data, dims) != 0) {
        *err = std::string("Error while 'Writing a snapshot': ") + custen_h5_last_error();
        return false;
    }
    ++r.snaps;
    return true;
}

// Take a resident request out of the run as failed: release its memory, record why.
static int drop(Server* S, int id, const std::string& why, double now) {
    Request& r = S->reqs[id];
    for (double* p : {r.g.buf[0], r.g.buf[1], r.g.tmp, r.g.ends, r.g.hbuf}) SRV_TRY(cudaFreeAsync(p, S->stream), "Freeing a grid");
    S->used -= (double)r.bytes;
    TableRef& t = S->tables[r.table_key];
    if (--t.refs == 0) {
        SRV_TRY(cudaFreeAsync(t.ptr, S->stream), "Freeing a table");
        S->used -= (double)t.bytes;
        t.ptr = nullptr;
    }
    r.state = 3;
    r.error = why;
    r.done_t = now;
    ++S->failed;
    return 0;
}

static int enqueue_steps(Server* S, int k) {
    for (int s = 0; s < k; ++s) {
        SRV_TRY(cudaMemsetAsync(S->counters, 0, kChCounters * sizeof(unsigned int), S->stream), "Resetting counters");
        // Fewer 32-line warps than FP64 sub-partitions (4 per SM): the sweeps are bound by a warp's own FP64
        // instruction count, so the y sweep's correction and update run as element-wise kernels. Every
        // configuration computes the same values, so a request's result does not depend on the choice.
        const ChConfig cfg = ch_config(S->n_rows < 4 * S->sms ? kChSplitConfig : kChBatchDefault);
        SRV_TRY(launch_ch_step(cfg, S->rhs_fp32 != 0, S->grids_d, S->items_rhs_d, S->n_rhs, S->items_rows_d,
                               S->n_rows, S->parity, S->counters, S->sms, S->stream),
                "Launching a step");
        S->launches += ch_launches_per_step(cfg);
        S->parity ^= 1;
    }
    return 0;
}

static int run(Server* S) {
    using clk = std::chrono::steady_clock;
    const auto t0 = clk::now();
    auto now = [&]() { return std::chrono::duration<double>(clk::now() - t0).count(); };
    std::vector<int> order(S->reqs.size());
    for (size_t k = 0; k < order.size(); ++k) order[k] = (int)k;
    std::stable_sort(order.begin(), order.end(),
                     [&](int a, int b) { return S->reqs[a].arrival < S->reqs[b].arrival; });
    size_t next = 0;   // first request (in arrival order) not yet admitted
    S->total_steps = 0;
    S->total_pt_steps = 0.0;
    S->failed = 0;
    S->max_active = 0;
    S->max_used = S->used;
    int done = 0;
    const int total = (int)S->reqs.size();
    while (done < total) {
        bool changed = false;
        // admit arrived requests, first come first served, while their memory fits the budget
        while (next < order.size()) {
            Request& r = S->reqs[order[next]];
            if (r.state != 0) { ++next; continue; }
            if (r.arrival > now()) break;
            const double need = (double)grid_bytes(r.n);
            if (S->used + need > S->budget && !S->active.empty()) break;
            int st = admit(S, order[next], now());
            ++next;
            if (st == kAdmitFailed) {
                ++done;
                continue;
            }
            if (st) return st;
            changed = true;
        }
        if (S->active.empty()) {
            if (next < order.size()) {
                const double wait = S->reqs[order[next]].arrival - now();
                if (wait > 0) std::this_thread::sleep_for(std::chrono::duration<double>(std::min(wait, 0.05)));
            }
            continue;
        }
        if (changed) {
            int st = rebuild(S);
            if (st) return st;
        }
        S->max_active = std::max<int>(S->max_active, (int)S->active.size());
        S->max_used = std::max(S->max_used, S->used);
        int k = S->chunk;
        for (int id : S->active) {
            const Request& r = S->reqs[id];
            k = std::min(k, r.remaining);
            if (r.snap_every > 0) k = std::min(k, r.snap_every - r.done_steps % r.snap_every);
        }
        nvtxRangePushA("chunk");
        int st = enqueue_steps(S, k);
        if (st) return st;
        SRV_TRY(cudaStreamSynchronize(S->stream), "Running a chunk");
        nvtxRangePop();
        const double t_chunk = now();
        std::vector<int> still;
        bool retired = false;
        for (int id : S->active) {
            Request& r = S->reqs[id];
            r.remaining -= k;
            r.done_steps += k;
            const double dt = S->dt_factor * (r.lx / r.n);   // dx = lx / n, dt = dt_factor * dx
            for (int q = 0; q < k; ++q) r.time += dt;
            S->total_steps += k;
            S->total_pt_steps += (double)k * r.n * r.n;
            if (r.snap_every > 0 && r.done_steps % r.snap_every == 0) {
                nvtxRangePushA("snapshot");
                std::string err;
                const bool ok = write_snapshot(S, r, &err);
                nvtxRangePop();
                if (!ok) {
                    if ((st = drop(S, id, err, t_chunk))) return st;
                    ++done;
                    retired = true;
                    continue;
                }
            }
            if (r.remaining == 0) {
                nvtxRangePushA("retire");
                st = retire(S, id, t_chunk);
                nvtxRangePop();
                if (st) return st;
                ++done;
                retired = true;
            } else {
                still.push_back(id);
            }
        }
        S->active.swap(still);
        if (retired && !S->active.empty()) {
            st = rebuild(S);
            if (st) return st;
        }
    }
    S->makespan = now();
    return 0;
}

}  // namespace ch
}  // namespace custen

using namespace custen::ch;

extern "C" {

const char* custen_ch_server_last_error(void) { return g_srv_err.c_str(); }

int custen_ch_server_create(void** out, double hbm_budget_bytes, int rhs_dtype, double gamma, double dt_factor,
                            int chunk_steps, int keep_results) {
    if (!out || hbm_budget_bytes <= 0 || chunk_steps < 1) return srv_arg("invalid arguments");
    Server* S = new Server();
    cudaGetDevice(&S->device);
    cudaDeviceGetAttribute(&S->sms, cudaDevAttrMultiProcessorCount, S->device);
    S->budget = hbm_budget_bytes;
    S->rhs_fp32 = rhs_dtype == CUSTEN_F32;
    S->gamma = gamma;
    S->dt_factor = dt_factor;
    S->chunk = chunk_steps;
    S->keep_results = keep_results;
    cudaError_t e = cudaStreamCreateWithFlags(&S->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMallocAsync(&S->counters, kChCounters * sizeof(unsigned int), S->stream);
    if (e == cudaSuccess) e = cudaMallocAsync(&S->mass_d, sizeof(double), S->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(S->stream);
    if (e != cudaSuccess) {
        delete S;
        return srv_fail(e, "Creating the server");
    }
    *out = S;
    return 0;
}

// Queue a request: an n x n grid of side lx advanced `steps` steps, arriving `arrival` seconds after
// the start of the run. c0: host initial field (n*n doubles), or NULL to draw U(-0.1, 0.1) from seed.
int custen_ch_server_submit(void* h, int n, double lx, int steps, const double* c0, unsigned long long seed,
                            double arrival, int* req_id) {
    Server* S = static_cast<Server*>(h);
    if (!S || n < 64 || n % BLK != 0 || steps < 1) return srv_arg("invalid request (n: multiple of 32, >= 64)");
    const double need = (double)grid_bytes(n) + (double)tab_size(n) * sizeof(double);
    if (need > S->budget)
        return srv_arg("request of n = " + std::to_string(n) + " needs " + std::to_string((long long)need) +
                       " bytes, above the server's HBM budget of " + std::to_string((long long)S->budget));
    Request r;
    r.n = n;
    r.lx = lx > 0 ? lx : 2.0 * M_PI;
    r.steps = steps;
    r.arrival = arrival;
    r.seed = seed;
    if (c0) r.c0.assign(c0, c0 + (size_t)n * n);
    S->reqs.push_back(std::move(r));
    if (req_id) *req_id = (int)S->reqs.size() - 1;
    return 0;
}

int custen_ch_server_run(void* h) {
    Server* S = static_cast<Server*>(h);
    if (!S) return srv_arg("invalid server");
    cudaSetDevice(S->device);
    return run(S);
}

// Per-request outcome: times on the server clock (seconds), means of the initial and final fields
// (compensated sums), and the final field when results are kept (c_out may be NULL).
int custen_ch_server_result(void* h, int id, double* c_out, double* arrival, double* admit_t, double* done_t,
                            double* mean0, double* mean_end) {
    Server* S = static_cast<Server*>(h);
    if (!S || id < 0 || id >= (int)S->reqs.size()) return srv_arg("invalid request id");
    const Request& r = S->reqs[id];
    if (r.state == 3) {
        g_srv_err = "request failed: " + r.error;
        return 3;
    }
    if (r.state != 2) return srv_arg("request not completed");
    if (c_out) {
        if (r.result.empty()) return srv_arg("results were not kept");
        memcpy(c_out, r.result.data(), r.result.size() * sizeof(double));
    }
    if (arrival) *arrival = r.arrival;
    if (admit_t) *admit_t = r.admit_t;
    if (done_t) *done_t = r.done_t;
    if (mean0) *mean0 = r.mean0;
    if (mean_end) *mean_end = r.mean_end;
    return 0;
}

// Periodic snapshots of a request (before run): every `every` steps (0: none) its state is written to
// dir/cahn_hilliard_<time %0.10f>.nc, the reference's Print_Out file (cuPentCahnADI.cu:103-140,
// 585-595) with "c_old" and "t" added; chunks end on those steps. A failed write fails the request.
int custen_ch_server_set_snapshots(void* h, int id, int every, const char* dir) {
    Server* S = static_cast<Server*>(h);
    if (!S || id < 0 || id >= (int)S->reqs.size() || every < 0 || (every > 0 && (!dir || !dir[0])))
        return srv_arg("invalid arguments");
    if (S->reqs[id].state != 0) return srv_arg("request already started");
    S->reqs[id].snap_every = every;
    S->reqs[id].snap_dir = every > 0 ? dir : "";
    return 0;
}

// Queue a request resumed from a snapshot: the grid and cCurr from "c" (n x n), cOld from "c_old" when
// present (else cCurr, a fresh start as in the reference), the simulated time from "t" (else 0); it
// advances `steps` more steps. A snapshot this server wrote resumes bit for bit.
int custen_ch_server_submit_snapshot(void* h, const char* path, double lx, int steps, double arrival, int* req_id) {
    Server* S = static_cast<Server*>(h);
    if (!S || !path) return srv_arg("invalid arguments");
    long long dims[2] = {0, 0};
    if (custen_h5_read(path, "c", nullptr, 0, dims) != 0) return srv_arg(std::string("Reading the snapshot: ") + custen_h5_last_error());
    if (dims[0] != dims[1] || dims[0] > (1 << 20)) return srv_arg("snapshot field is not a square grid");
    const int n = (int)dims[0];
    std::vector<double> c((size_t)n * n), old;
    if (custen_h5_read(path, "c", c.data(), (long long)c.size(), dims) != 0)
        return srv_arg(std::string("Reading the snapshot: ") + custen_h5_last_error());
    long long od[2];
    if (custen_h5_read(path, "c_old", nullptr, 0, od) == 0) {
        if (od[0] != n || od[1] != n) return srv_arg("snapshot c_old does not match c");
        old.resize(c.size());
        if (custen_h5_read(path, "c_old", old.data(), (long long)old.size(), od) != 0)
            return srv_arg(std::string("Reading the snapshot: ") + custen_h5_last_error());
    }
    double t = 0.0;
    long long td[2];
    if (custen_h5_read(path, "t", nullptr, 0, td) == 0 && td[0] * td[1] == 1) custen_h5_read(path, "t", &t, 1, td);
    int id = -1;
    const int st = custen_ch_server_submit(h, n, lx, steps, c.data(), 0, arrival, &id);
    if (st) return st;
    S->reqs[id].c_old0 = std::move(old);
    S->reqs[id].time = t;
    if (req_id) *req_id = id;
    return 0;
}

// Snapshots a request has written so far.
int custen_ch_server_snapshots_written(void* h, int id, int* count) {
    Server* S = static_cast<Server*>(h);
    if (!S || id < 0 || id >= (int)S->reqs.size() || !count) return srv_arg("invalid arguments");
    *count = S->reqs[id].snaps;
    return 0;
}

// State of a request: 0 pending, 1 resident, 2 done, 3 failed (custen_ch_server_result reports why).
int custen_ch_server_request_state(void* h, int id, int* state) {
    Server* S = static_cast<Server*>(h);
    if (!S || id < 0 || id >= (int)S->reqs.size() || !state) return srv_arg("invalid arguments");
    *state = S->reqs[id].state;
    return 0;
}

// Test hook for failure isolation: kind 1 makes the request's device allocation at admission fail with
// cudaErrorMemoryAllocation (a fake of the failing call, on the host; nothing reaches the GPU).
int custen_ch_server_inject_failure(void* h, int id, int kind) {
    Server* S = static_cast<Server*>(h);
    if (!S || id < 0 || id >= (int)S->reqs.size() || kind < 0 || kind > 1) return srv_arg("invalid arguments");
    S->reqs[id].inject = kind;
    return 0;
}

// stats: makespan (s), total steps, total point-steps, largest resident set, peak resident bytes,
// kernel launches.
int custen_ch_server_stats(void* h, double* makespan, long long* total_steps, double* total_pt_steps, int* max_active,
                           double* peak_bytes, unsigned long long* launches) {
    Server* S = static_cast<Server*>(h);
    if (!S) return srv_arg("invalid server");
    if (makespan) *makespan = S->makespan;
    if (total_steps) *total_steps = S->total_steps;
    if (total_pt_steps) *total_pt_steps = S->total_pt_steps;
    if (max_active) *max_active = S->max_active;
    if (peak_bytes) *peak_bytes = S->max_used;
    if (launches) *launches = S->launches;
    return 0;
}

int custen_ch_server_destroy(void* h) {
    Server* S = static_cast<Server*>(h);
    if (!S) return 0;
    cudaStreamSynchronize(S->stream);
    for (int id : S->active) {
        Request& r = S->reqs[id];
        for (double* p : {r.g.buf[0], r.g.buf[1], r.g.tmp, r.g.ends, r.g.hbuf}) cudaFreeAsync(p, S->stream);
    }
    for (auto& t : S->tables)
        if (t.second.ptr) cudaFreeAsync(t.second.ptr, S->stream);
    if (S->grids_d) cudaFreeAsync(S->grids_d, S->stream);
    if (S->items_rhs_d) cudaFreeAsync(S->items_rhs_d, S->stream);
    if (S->items_rows_d) cudaFreeAsync(S->items_rows_d, S->stream);
    cudaFreeAsync(S->counters, S->stream);
    cudaFreeAsync(S->mass_d, S->stream);
    cudaStreamSynchronize(S->stream);
    cudaStreamDestroy(S->stream);
    delete S;
    return 0;
}

}  // extern "C"
