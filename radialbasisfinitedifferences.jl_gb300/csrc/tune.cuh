// Autotuner of the weight-solve launches (tune.cu): per shape class of local systems, the
// kernel (FP64, register Schur mixed, shared-memory mixed) and its warps per CTA, chosen by
// timing candidate launches on a sample of the class's systems and cached on the handle.
#pragma once

#include <string>
#include <vector>

#include "rbffd_internal.cuh"

enum { SOLVE_KERNEL_FP64 = 0, SOLVE_KERNEL_SCHUR = 1, SOLVE_KERNEL_SMEM_MIXED = 2 };

struct SolveConfig {
    int kernel = SOLVE_KERNEL_FP64;
    int wpb = 4;
};

struct TuneRecord {
    int precision, max_n, max_m, nops, p, unscaled, collocated;
    SolveConfig cfg;
    bool measured;                 // false: heuristic choice (class too small to time)
    int64_t sample;                // systems per timed candidate launch
    std::vector<SolveConfig> cand; // candidates timed, in order
    std::vector<float> ms;         // their times on the sample
};

class SolveTuner {
public:
    // The configuration for the systems of `a` (one shape class: a.max_n, a.max_m bound them).
    // On a class seen for the first time with enough systems, times every candidate on stream
    // st on tune_sample_systems() systems spread evenly over the class, listed in sample_list
    // (device scratch of that many entries; their weights are written and later rewritten
    // identically by the real launch; the refinement histogram, fallback queue and claim
    // counter of `a` are cleared afterwards).  fixed_wpb > 0 pins the warps per CTA (no timing).
    cudaError_t choose(const SolveArgs &a, const OpTable &t, int precision, int fixed_wpb, int num_sms,
                       int32_t *sample_list, cudaStream_t st, SolveConfig *out);
    std::string report() const;

private:
    std::vector<TuneRecord> cache_;
};

// Systems per timed candidate launch.
inline int64_t tune_sample_systems(int num_sms) { return (int64_t)num_sms * 64; }

// One launch of the solve kernel `c` over the systems of `a`.
cudaError_t launch_solve_config(const SolveArgs &a, const OpTable &t, SolveConfig c, int num_sms, cudaStream_t st);
