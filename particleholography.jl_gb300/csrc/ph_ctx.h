// ph_ctx.h -- the context object behind the opaque ph_ctx handle.
#pragma once

#include <cuda_runtime.h>

#include <atomic>
#include <cstdint>
#include <list>
#include <map>
#include <mutex>
#include <string>
#include <unordered_map>
#include <vector>


struct ph_graph_entry {
    std::string key;
    cudaGraphExec_t exec = nullptr;
    int64_t kernels = 0;   // kernels launched by one replay
};

// Reconstruction knobs the autotuner chose for one (n_fast, n_slow).
struct ph_tuning {
    int form = 0;           // PH_FORM_* of the projection's row pass (used under PH_FORM_TUNED)
    int group_cap = 0;      // slices per pass A / pass B CTA at most (0 = the built-in rule)
    int batch_slices = 0;   // slices per batch of intermediates (0 = the built-in rule)
    int slices = 0;         // slices of the workload it was timed on
    double ms = 0.0;        // its time per reconstruction
};

struct ph_prof_record {
    const char *name;
    cudaEvent_t start, stop;
};

struct ph_ctx {
    int device = 0;
    size_t budget = 0;              // 0 = unbounded
    std::mutex mu;
    std::string err;

    // twiddle tables W_N^i, i in [0, N), one per transform length
    std::unordered_map<int, float2 *> tw;

    // tables of the split-precision tensor-core pass (DFT matrices, twiddles),
    // one per (length, form): key 8 n + form
    std::unordered_map<int, void *> tc_tables;

    // scratch arena (grown on demand, never shrunk until destroy)
    void *scratch = nullptr;
    size_t scratch_bytes = 0;

    // unit vectors (cos, sin)(2 pi j / 4096) in FP64 for the spectrum's phase rates
    float4 *phase_tab = nullptr;

    // small fixed device area: [0] loop-limit error flag (int), [8..) 4 doubles of accumulators
    void *small = nullptr;

    // stream ordering between calls on different streams
    cudaStream_t last_stream = nullptr;
    bool has_last = false;
    cudaEvent_t done = nullptr;

    // private stream used only to record CUDA graphs
    cudaStream_t capture_stream = nullptr;
    std::list<ph_graph_entry> graphs;   // most recently used first

    std::atomic<int64_t> launches{0};

    int64_t opt_slice_batch = 0;
    int64_t opt_use_graphs = 1;
    int64_t opt_loop_limit = int64_t(1) << 20;
    int64_t opt_profile = 0;
    int64_t opt_form = 0;           // PH_FORM_*: arithmetic of the projection's row pass
    std::map<std::pair<int, int>, ph_tuning> tuned;   // (n_fast, n_slow) -> autotuner's choice

    // profiler: pending event pairs and a pool of spare events
    std::vector<ph_prof_record> prof;
    std::vector<cudaEvent_t> prof_pool;
};
