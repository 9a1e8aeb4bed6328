// vpf_tune.cu -- autotuner of the step's launch configuration (abm_vpf_autotune).
//
// Every form of the step (group form with automatic or 1-16 neighbour chunks, L1 form with 1, 2 or 4 warps
// per focal agent and 1-16 neighbour chunks, tiled form with several agents-per-block and tile
// lengths) gives bit-identical
// results, so the best one for a workload is an empirical question: the tuner times each
// candidate on the caller's own state and stream and applies the fastest.
#include <vector>

#include "../../include/abm_vpf.h"
#include "vpf_host.h"

namespace abm {

static std::vector<abm_step_config> tune_candidates(bool segmented) {
    std::vector<abm_step_config> c;
    const int wpas[] = {1, 2, 4};
    if (segmented) {
        c.push_back({3, 1, 1, 8, 8192, -1.f});   // group form (if it applies)
        for (int wpa : wpas) c.push_back({1, wpa, 1, 8, 8192, -1.f});
        return c;
    }
    const int chunks[] = {1, 2, 4, 8, 16};
    // group form (if it applies): the automatic chunks (with the decreasing round-major plan
    // beyond one wave of blocks), then 1-16 equal chunks
    c.push_back({3, 1, 0, 8, 8192, -1.f});
    for (int ch : chunks) c.push_back({3, 1, ch, 8, 8192, -1.f});
    for (int wpa : wpas)
        for (int ch : chunks) c.push_back({1, wpa, ch, 8, 8192, -1.f});
    const int warps[] = {4, 8, 16};
    const int tiles[] = {1024, 2048, 4096, 8192};
    for (int w : warps)
        for (int t : tiles) c.push_back({2, 1, 1, w, t, -1.f});
    return c;
}

static void apply_config(const abm_step_config &c) {
    abm_vpf_set_step_mode(c.mode, c.warps_per_agent);
    abm_vpf_set_step_config(c.warps_per_block, c.tile);
    abm_vpf_set_step_split(c.chunks);
}

}  // namespace abm

using namespace abm;

extern "C" int abm_vpf_autotune(const abm_swarm_state *in, int32_t n, const int32_t *seg_begin_dev,
                                const int32_t *seg_end_dev, const int32_t *order_dev,
                                const abm_vf_params *p, const abm_agent_overrides *ov,
                                int32_t reps, abm_step_config *best, abm_step_config *tried,
                                int32_t max_tried, int32_t *n_tried, void *stream) {
    const char *fn = "abm_vpf_autotune";
    if (!in || !p || !best) return set_error(ABM_ERR_INVALID_ARG, "%s: NULL argument", fn);
    if (n <= 0) return set_error(ABM_ERR_INVALID_ARG, "%s: n=%d", fn, n);
    if (reps < 1 || reps > 1000) return set_error(ABM_ERR_INVALID_ARG, "%s: reps=%d", fn, reps);
    if ((seg_begin_dev == nullptr) != (seg_end_dev == nullptr))
        return set_error(ABM_ERR_INVALID_ARG, "%s: give both segment arrays or neither", fn);
    if (max_tried < 0 || (max_tried > 0 && !tried))
        return set_error(ABM_ERR_INVALID_ARG, "%s: tried is NULL", fn);
    const bool segmented = seg_begin_dev != nullptr;
    cudaStream_t s = (cudaStream_t)stream;
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    int st = check_cuda(cudaStreamIsCapturing(s, &cap), "cudaStreamIsCapturing");
    if (st) return st;
    if (cap != cudaStreamCaptureStatusNone)
        return set_error(ABM_ERR_INVALID_ARG, "%s: stream is capturing", fn);

    // the current configuration, restored if every candidate fails
    abm_step_config saved{};
    abm_vpf_get_step_mode(&saved.mode, &saved.warps_per_agent);
    abm_vpf_get_step_config(&saved.warps_per_block, &saved.tile);
    abm_vpf_get_step_split(&saved.chunks);

    float *scratch = nullptr;
    st = check_cuda(cudaMalloc((void **)&scratch, 4 * sizeof(float) * (size_t)n),
                    "cudaMalloc(tuner scratch)");
    if (st) return st;
    abm_swarm_state out{scratch, scratch + n, scratch + 2 * (size_t)n, scratch + 3 * (size_t)n};
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    st = check_cuda(cudaEventCreate(&e0), "cudaEventCreate");
    if (!st) st = check_cuda(cudaEventCreate(&e1), "cudaEventCreate");

    auto step = [&]() -> int {
        return segmented ? abm_vpf_flock_batched(in, &out, n, seg_begin_dev, seg_end_dev,
                                                 order_dev, p, ov, nullptr, nullptr, nullptr,
                                                 stream)
                         : abm_vpf_flock_step(in, &out, n, p, ov, nullptr, nullptr, nullptr,
                                              stream);
    };
    std::vector<abm_step_config> cand = tune_candidates(segmented);
    int best_k = -1;
    for (size_t k = 0; k < cand.size() && !st; ++k) {
        abm_step_config &c = cand[k];
        apply_config(c);
        int r = step();   // untimed: tables, workspace, first-touch
        if (r < 0) {      // this form is refused for the workload (e.g. Rv too large)
            c.ms_per_step = -1.f;
            continue;
        }
        cudaEventRecord(e0, s);
        for (int i = 0; i < reps && r >= 0; ++i) r = step();
        cudaEventRecord(e1, s);
        st = check_cuda(cudaEventSynchronize(e1), "tuner timing");
        if (st) break;
        if (r < 0) {
            c.ms_per_step = -1.f;
            continue;
        }
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        c.ms_per_step = ms / (float)reps;
        if (best_k < 0 || c.ms_per_step < cand[best_k].ms_per_step) best_k = (int)k;
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    cudaFree(scratch);
    if (n_tried) *n_tried = (int32_t)cand.size();
    for (int k = 0; k < max_tried && k < (int)cand.size(); ++k) tried[k] = cand[k];
    if (st || best_k < 0) {
        apply_config(saved);
        return st ? st : set_error(ABM_ERR_UNSUPPORTED, "%s: no configuration ran", fn);
    }
    *best = cand[best_k];
    apply_config(*best);
    return ABM_OK;
}
