// Autotuner of the batched weight solves: which kernel and how many warps per CTA for each
// shape class of local systems (stencil size, number of monomials, number of operators).
//
// The candidates differ in occupancy and in how the per-warp shared memory and registers are
// spent, and which one wins depends on the class: the register Schur kernel (mixed precision,
// n <= 64, m <= 32, at most 8 operators) against the shared-memory mixed kernel, and the warps
// per CTA of each (the per-warp shared memory grows with s = n + m, so a wide CTA can leave an
// SM's shared memory partly unused).  In mixed precision the FP64 kernel is a candidate too: a
// class of ill-conditioned systems (PHS r^5 with high-degree polynomials) can need so many
// refinement steps that solving it directly in FP64 is faster, and its weights are at least as
// accurate.  Each candidate is launched once on a few warm-up systems (module load) and then
// timed with CUDA events on `sample` systems spread evenly over the class (the first systems of
// a class are the nodes of one edge of the domain, whose conditioning is not the class's); the
// fastest is cached on the handle for that class, so later builds pay nothing.
#include <stdint.h>
#include <stdio.h>
#include <string.h>

#include "tune.cuh"

namespace {

bool schur_eligible(const SolveArgs &a, const OpTable &t)
{
    return t.nops <= 8 && a.max_n <= 64 && a.max_m <= 32 && !a.unscaled_overload;
}

size_t smem_optin()
{
    int dev = 0, v = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    return (size_t)v;
}

// Largest CTA (<= 8 warps) whose shared memory still lets >= 2 CTAs share an SM.
int heuristic_wpb(size_t per_warp)
{
    const size_t budget = 110 * 1024;
    int w = 8;
    while (w > 1 && per_warp * w > budget) w >>= 1;
    return w;
}

std::vector<SolveConfig> candidates(const SolveArgs &a, const OpTable &t, int precision)
{
    std::vector<SolveConfig> c;
    const size_t cap = smem_optin();
    if (precision == RBFFD_PREC_FP64) {
        const size_t pw = solve_fp64_smem_per_warp(a.max_s, a.max_n, t.nops);
        for (int w : {1, 2, 4, 8})
            if (pw * w <= cap) c.push_back({SOLVE_KERNEL_FP64, w});
        return c;
    }
    // the Schur kernel starts a CTA's systems together (instruction-cache locality), so its
    // candidates are CTAs of several warps, up to all of an SM's resident warps
    if (schur_eligible(a, t))
        for (int w : {4, 8, 16})
            if (w <= (a.max_n <= 32 ? 16 : 8)) c.push_back({SOLVE_KERNEL_SCHUR, w});
    const size_t pw = solve_mixed_smem_per_warp(a.max_s, a.max_n, t.nops);
    for (int w : {1, 2, 4, 8})
        if (pw * w <= cap) c.push_back({SOLVE_KERNEL_SMEM_MIXED, w});
    const size_t pf = solve_fp64_smem_per_warp(a.max_s, a.max_n, t.nops);
    for (int w : {1, 2, 4, 8})
        if (pf * w <= cap) c.push_back({SOLVE_KERNEL_FP64, w});
    return c;
}

SolveConfig heuristic(const SolveArgs &a, const OpTable &t, int precision, int fixed_wpb)
{
    if (precision == RBFFD_PREC_FP64) {
        const int w = fixed_wpb > 0 ? fixed_wpb : heuristic_wpb(solve_fp64_smem_per_warp(a.max_s, a.max_n, t.nops));
        return {SOLVE_KERNEL_FP64, w};
    }
    if (schur_eligible(a, t)) return {SOLVE_KERNEL_SCHUR, fixed_wpb > 0 && fixed_wpb <= 16 ? fixed_wpb : 4};
    const int w = fixed_wpb > 0 ? fixed_wpb : heuristic_wpb(solve_mixed_smem_per_warp(a.max_s, a.max_n, t.nops));
    return {SOLVE_KERNEL_SMEM_MIXED, w};
}

// out[i] = the class's system at position floor(i * nsys / sample) (list[...] when the class is a
// list of systems, base + the position otherwise).
__global__ void sample_list_kernel(const int32_t *list, int64_t base, int64_t nsys, int64_t sample, int32_t *out)
{
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= sample) return;
    const int64_t pos = i * nsys / sample;
    out[i] = list ? list[pos] : (int32_t)(base + pos);
}

const char *kernel_name(int k)
{
    return k == SOLVE_KERNEL_FP64 ? "fp64" : k == SOLVE_KERNEL_SCHUR ? "schur" : "smem-mixed";
}

}  // namespace

cudaError_t launch_solve_config(const SolveArgs &a, const OpTable &t, SolveConfig c, int num_sms, cudaStream_t st)
{
    switch (c.kernel) {
    case SOLVE_KERNEL_FP64: return launch_solve_fp64(a, t, c.wpb, num_sms, st);
    case SOLVE_KERNEL_SCHUR: return launch_solve_mixed_reg(a, t, a.max_m, c.wpb, num_sms, st);
    default: return launch_solve_mixed(a, t, c.wpb, num_sms, st);
    }
}

cudaError_t SolveTuner::choose(const SolveArgs &a, const OpTable &t, int precision, int fixed_wpb, int num_sms,
                               int32_t *sample_list, cudaStream_t st, SolveConfig *out)
{
    const int collocated = a.Y == nullptr;
    for (const TuneRecord &r : cache_)
        if (r.precision == precision && r.max_n == a.max_n && r.max_m == a.max_m && r.nops == t.nops && r.p == t.p &&
            r.unscaled == a.unscaled_overload && r.collocated == collocated) {
            *out = r.cfg;
            return cudaSuccess;
        }
    TuneRecord rec{precision, a.max_n, a.max_m, t.nops, t.p, a.unscaled_overload, collocated, {}, false, 0, {}, {}};
    // enough systems to fill every SM a few times over
    const int64_t sample = tune_sample_systems(num_sms);
    std::vector<SolveConfig> cand = candidates(a, t, precision);
    if (fixed_wpb > 0 || a.nsys < 3 * sample || a.sys_base + a.nsys > INT32_MAX || cand.size() < 2 || !a.next_sys ||
        !sample_list) {
        // a small class is not cached: a later, larger class of the same shape may be timed
        *out = heuristic(a, t, precision, fixed_wpb);
        return cudaSuccess;
    }
    sample_list_kernel<<<(unsigned)((sample + 255) / 256), 256, 0, st>>>(a.sys_list, a.sys_base, a.nsys, sample,
                                                                         sample_list);
    cudaError_t lerr = cudaGetLastError();
    if (lerr != cudaSuccess) return lerr;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    float best = 1e30f;
    SolveConfig win = cand[0];
    cudaError_t err = cudaSuccess;
    for (const SolveConfig &c : cand) {
        SolveArgs s = a;
        s.sys_list = sample_list;
        s.nsys = 32;  // warm-up: module load and first-launch costs stay out of the timing
        if ((err = cudaMemsetAsync(a.next_sys, 0, sizeof(unsigned long long), st)) != cudaSuccess) break;
        err = launch_solve_config(s, t, c, num_sms, st);
        if (err == cudaErrorNotSupported) {  // a shape this kernel does not take after all
            cudaGetLastError();
            err = cudaSuccess;
            continue;
        }
        if (err != cudaSuccess) break;
        s.nsys = sample;
        if ((err = cudaMemsetAsync(a.next_sys, 0, sizeof(unsigned long long), st)) != cudaSuccess) break;
        cudaEventRecord(e0, st);
        if ((err = launch_solve_config(s, t, c, num_sms, st)) != cudaSuccess) break;
        cudaEventRecord(e1, st);
        if ((err = cudaEventSynchronize(e1)) != cudaSuccess) break;
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, e0, e1);
        rec.cand.push_back(c);
        rec.ms.push_back(ms);
        if (ms < best) {
            best = ms;
            win = c;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (err != cudaSuccess) return err;
    // Among Schur configurations within 1.5 % of the fastest, the widest CTA: its warps start
    // their systems together, which keeps them in the same part of the kernel over a long
    // launch, an advantage a short sample does not show (1,048,576 30-node systems: 8 warps
    // per CTA 42.9 ms, 4 warps 43.4 ms, tied at 0.420 ms on the sample).
    if (win.kernel == SOLVE_KERNEL_SCHUR)
        for (size_t i = 0; i < rec.cand.size(); i++)
            if (rec.cand[i].kernel == SOLVE_KERNEL_SCHUR && rec.ms[i] <= best * 1.015f && rec.cand[i].wpb > win.wpb)
                win = rec.cand[i];
    // the sample systems are solved again by the real launch: clear what they counted
    if (a.fallback_count && (err = cudaMemsetAsync(a.fallback_count, 0, sizeof(int), st)) != cudaSuccess) return err;
    if (a.hist && (err = cudaMemsetAsync(a.hist, 0, 8 * sizeof(unsigned long long), st)) != cudaSuccess) return err;
    if ((err = cudaMemsetAsync(a.next_sys, 0, sizeof(unsigned long long), st)) != cudaSuccess) return err;
    rec.cfg = rec.cand.empty() ? heuristic(a, t, precision, 0) : win;
    rec.measured = !rec.cand.empty();
    rec.sample = sample;
    cache_.push_back(rec);
    *out = rec.cfg;
    return cudaSuccess;
}

std::string SolveTuner::report() const
{
    std::string s;
    char buf[256];
    for (const TuneRecord &r : cache_) {
        snprintf(buf, sizeof(buf), "%s n<=%d m<=%d ops=%d p=%d%s: %s x%d warps", r.precision ? "mixed" : "fp64",
                 r.max_n, r.max_m, r.nops, r.p, r.collocated ? "" : " (Y!=X)", kernel_name(r.cfg.kernel), r.cfg.wpb);
        s += buf;
        if (r.measured) {
            s += " (timed on " + std::to_string(r.sample) + " systems:";
            for (size_t i = 0; i < r.cand.size(); i++) {
                snprintf(buf, sizeof(buf), " %s x%d %.3f ms", kernel_name(r.cand[i].kernel), r.cand[i].wpb, r.ms[i]);
                s += buf;
                if (i + 1 < r.cand.size()) s += ",";
            }
            s += ")";
        }
        s += "\n";
    }
    return s;
}
