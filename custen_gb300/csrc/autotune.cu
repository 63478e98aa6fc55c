// Autotuner for the stencil kernels: picks the tile configuration (stencil_configs.h) of a launch
// geometry by timing every configuration on the launch itself, and caches the choice in a JSON file.
//
// Key: GPU name | variant | dtype | nx x rows | window H.L.R.V.T.B | fused cube | aligned rows. Every
// configuration computes identical values (same FMA chain per point), so tuning on the caller's own
// buffers is safe: the last timed launch leaves the correct output.
//
// Modes (custen_set_autotune, or the CUSTEN_AUTOTUNE environment variable at first use):
//   0  look the key up in the cache; default configuration when absent (the default mode)
//   1  as 0, and tune keys that are absent (at the handle's first Compute), then store them
//   2  tune every new handle, overwriting the cache entry
// Cache file: custen_set_tune_cache(path), else CUSTEN_TUNE_CACHE, else
// $HOME/.cache/custen_gb300/tune.json. Tuning is skipped while the stream is being captured.
#include <cuda_runtime.h>

#include <cerrno>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <sys/stat.h>
#include <unistd.h>
#include <vector>

#include "stencil_configs.h"

namespace custen {
namespace {

std::mutex g_mu;
bool g_loaded = false;
int g_mode = -1;                   // -1: not yet read from the environment
std::string g_path;                // empty: default
struct Entry {
    std::string config;
    int index;
    std::vector<float> ms;
};
std::map<std::string, Entry> g_cache;

std::string default_path() {
    if (const char* e = getenv("CUSTEN_TUNE_CACHE")) {
        if (*e) return e;
    }
    const char* home = getenv("HOME");
    return std::string(home && *home ? home : "/tmp") + "/.cache/custen_gb300/tune.json";
}

const std::string& cache_path() {
    if (g_path.empty()) g_path = default_path();
    return g_path;
}

int mode() {
    if (g_mode < 0) {
        const char* e = getenv("CUSTEN_AUTOTUNE");
        g_mode = (e && *e) ? atoi(e) : 0;
        if (g_mode < 0 || g_mode > 2) g_mode = 0;
    }
    return g_mode;
}

// The file holds one entry per line: "key": {"config": "name", "index": k, "ms": [...]}
void load() {
    if (g_loaded) return;
    g_loaded = true;
    FILE* f = fopen(cache_path().c_str(), "r");
    if (!f) return;
    char line[4096];
    while (fgets(line, sizeof(line), f)) {
        const char* q0 = strchr(line, '"');
        if (!q0) continue;
        const char* q1 = strchr(q0 + 1, '"');
        if (!q1) continue;
        std::string key(q0 + 1, q1 - q0 - 1);
        const char* c = strstr(q1, "\"config\": \"");
        const char* ix = strstr(q1, "\"index\": ");
        if (!c || !ix) continue;
        c += strlen("\"config\": \"");
        const char* ce = strchr(c, '"');
        if (!ce) continue;
        Entry en;
        en.config.assign(c, ce - c);
        en.index = atoi(ix + strlen("\"index\": "));
        const int dtype = en.config.compare(0, 4, "f64_") == 0 ? DT_F64 : DT_F32;
        // entries written for another configuration table are ignored
        if (en.index < 0 || en.index >= kNumConfigs || en.config != config_name(dtype, en.index)) continue;
        g_cache[key] = en;
    }
    fclose(f);
}

void mkdirs(const std::string& path) {
    for (size_t p = path.find('/', 1); p != std::string::npos; p = path.find('/', p + 1)) {
        std::string d = path.substr(0, p);
        if (mkdir(d.c_str(), 0755) != 0 && errno != EEXIST) return;
    }
}

void save() {
    const std::string& path = cache_path();
    mkdirs(path);
    // a per-process temporary, renamed over the cache: concurrent writers never interleave
    const std::string tmp = path + "." + std::to_string((long long)getpid()) + ".tmp";
    FILE* f = fopen(tmp.c_str(), "w");
    if (!f) return;
    fprintf(f, "{\n\"custen_gb300_tune_cache\": 1,\n\"entries\": {\n");
    size_t k = 0;
    for (const auto& kv : g_cache) {
        fprintf(f, "\"%s\": {\"config\": \"%s\", \"index\": %d, \"ms\": [", kv.first.c_str(), kv.second.config.c_str(),
                kv.second.index);
        for (size_t i = 0; i < kv.second.ms.size(); ++i) fprintf(f, "%s%.5f", i ? ", " : "", kv.second.ms[i]);
        fprintf(f, "]}%s\n", ++k < g_cache.size() ? "," : "");
    }
    fprintf(f, "}\n}\n");
    if (fclose(f) != 0 || rename(tmp.c_str(), path.c_str()) != 0) remove(tmp.c_str());
}

std::string gpu_name() {
    static std::string names[64];
    static std::mutex mu;
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= 64) return "gpu";
    std::lock_guard<std::mutex> lock(mu);
    if (names[dev].empty()) {
        cudaDeviceProp prop;
        names[dev] = cudaGetDeviceProperties(&prop, dev) == cudaSuccess ? prop.name : "gpu";
        for (char& ch : names[dev])
            if (ch == '"' || ch == '|') ch = '_';
    }
    return names[dev];
}

std::string make_key(const StencilArgs& a, int dtype) {
    char buf[256];
    snprintf(buf, sizeof(buf), "|v%d|%s|%dx%d|%d.%d.%d.%d.%d.%d|pre%d|aligned%d", a.variant, dtype == DT_F64 ? "f64" : "f32",
             a.nx, a.rows, a.H, a.L, a.R, a.V, a.T, a.B, a.pre, a.vec_ok);
    return gpu_name() + buf;
}

// Time every configuration on this launch (one warm-up and `reps` timed launches each).
int tune(const StencilArgs& a, int dtype, cudaStream_t s, int reps, std::vector<float>* ms_out) {
    cudaEvent_t e0, e1;
    if (cudaEventCreate(&e0) != cudaSuccess) return -1;
    if (cudaEventCreate(&e1) != cudaSuccess) {
        cudaEventDestroy(e0);
        return -1;
    }
    int best = -1;
    float best_ms = 0.f;
    std::vector<float> ms(kNumConfigs, -1.f);
    for (int c = 0; c < kNumConfigs; ++c) {
        int path = 0;
        if (launch_stencil_cfg(a, dtype, c, s, &path) != cudaSuccess) {
            cudaGetLastError();
            continue;
        }
        cudaEventRecord(e0, s);
        bool ok = true;
        for (int r = 0; r < reps && ok; ++r) ok = launch_stencil_cfg(a, dtype, c, s, &path) == cudaSuccess;
        cudaEventRecord(e1, s);
        if (!ok || cudaEventSynchronize(e1) != cudaSuccess) {
            cudaGetLastError();
            continue;
        }
        float t = 0.f;
        cudaEventElapsedTime(&t, e0, e1);
        ms[c] = t / reps;
        if (best < 0 || ms[c] < best_ms) {
            best = c;
            best_ms = ms[c];
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (ms_out) *ms_out = ms;
    return best;
}

}  // namespace

// The configuration for a device-resident launch: from the cache, from tuning (modes 1, 2 or force),
// else the default. Returns the index.
int choose_config(const StencilArgs& a, int dtype, cudaStream_t s, bool force, int reps) {
    std::lock_guard<std::mutex> lock(g_mu);
    const int m = force ? 2 : mode();
    load();
    const std::string key = make_key(a, dtype);
    auto it = g_cache.find(key);
    if (m < 2 && it != g_cache.end()) return it->second.index;
    if (m == 0) return 0;
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(s, &cap) != cudaSuccess || cap != cudaStreamCaptureStatusNone) {
        cudaGetLastError();
        return it != g_cache.end() ? it->second.index : 0;
    }
    std::vector<float> ms;
    const int best = tune(a, dtype, s, reps > 0 ? reps : 3, &ms);
    if (best < 0) return 0;
    Entry en;
    en.config = config_name(dtype, best);
    en.index = best;
    en.ms = ms;
    g_cache[key] = en;
    save();
    return best;
}

void set_autotune_mode(int m) {
    std::lock_guard<std::mutex> lock(g_mu);
    g_mode = (m < 0 || m > 2) ? 0 : m;
}

void set_tune_cache(const char* path) {
    std::lock_guard<std::mutex> lock(g_mu);
    g_path = (path && *path) ? path : default_path();
    g_cache.clear();
    g_loaded = false;
}

std::string tune_cache_path() {
    std::lock_guard<std::mutex> lock(g_mu);
    return cache_path();
}

}  // namespace custen
