// sph_tune.cu -- the launch autotuner of the staged and persistent steps.
//
// It times a few steps of each candidate configuration on a saved copy of
// the state (restored after every trial, so the simulation does not move):
//   * the staged step graph with the density pass under each launch shape
//     (sph_shapes.cu: 128 threads x 7 CTAs per SM -- the default --, 64 x 14,
//     256 x 3, 128 x 6, 128 x 8), then the force pass under each shape with
//     the best density shape (coordinate descent: 1 + 4 + 4 trials);
//   * where allowed (batches), the persistent fused step at 1, 2, ... CTAs
//     per SM up to its occupancy limit.
// The fastest is kept.  Choices are cached per GPU (name, SM count) and size
// class (floor(log2) of the particle count and of the scene count, and the
// arithmetic), in the process and -- when SPH_AUTOTUNE_CACHE names a file --
// on disk, one line per entry, so a later run of the same class on the same
// GPU skips the trials.
#include "sph_state.h"

#include <cstdio>
#include <cstdlib>
#include <map>
#include <mutex>

namespace sph {
namespace {

std::mutex g_tune_mutex;
std::map<std::string, TuneChoice> g_tune_cache;
bool g_tune_file_loaded = false;

uint32_t ilog2(uint64_t v)
{
    uint32_t r = 0;
    while (v > 1) {
        v >>= 1;
        ++r;
    }
    return r;
}

void load_cache_file()
{
    if (g_tune_file_loaded) return;
    g_tune_file_loaded = true;
    const char* path = std::getenv("SPH_AUTOTUNE_CACHE");
    if (!path || !*path) return;
    FILE* f = std::fopen(path, "r");
    if (!f) return;
    char key[256];
    TuneChoice c{};
    int mode = 0;
    unsigned ctas = 0;
    while (std::fscanf(f, "%255s %d %u %d %d %f", key, &mode, &ctas, &c.density_shape, &c.force_shape, &c.ms) == 6) {
        c.mode = mode == 1 ? StepMode::Persistent : StepMode::Staged;
        c.ctas = ctas;
        if (c.density_shape >= 0 && c.density_shape < kShapeCount && c.force_shape >= 0 &&
            c.force_shape < kForceShapeCount)
            g_tune_cache[key] = c;
    }
    std::fclose(f);
}

void append_cache_file(const std::string& key, const TuneChoice& c)
{
    const char* path = std::getenv("SPH_AUTOTUNE_CACHE");
    if (!path || !*path) return;
    FILE* f = std::fopen(path, "a");
    if (!f) return;
    std::fprintf(f, "%s %d %u %d %d %.6f\n", key.c_str(), c.mode == StepMode::Persistent ? 1 : 0, c.ctas,
                 c.density_shape, c.force_shape, c.ms);
    std::fclose(f);
}

}  // namespace

std::string StepState::tune_key(bool allow_persistent) const
{
    cudaDeviceProp prop{};
    if (cudaGetDeviceProperties(&prop, device_) != cudaSuccess) prop.name[0] = 0;
    std::string name(prop.name);
    for (char& ch : name)
        if (ch == ' ') ch = '_';
    char buf[256];
    std::snprintf(buf, sizeof buf, "%s/sm%d/n%u/k%u/%s/%s", name.c_str(), prop.multiProcessorCount,
                  ilog2(total_n), ilog2(scenes.size()), exact_ ? "exact" : "fast",
                  allow_persistent ? "any" : "staged");
    return buf;
}

void StepState::apply_choice(const TuneChoice& c)
{
    set_shapes(c.density_shape, c.force_shape);
    set_persistent_ctas(c.mode == StepMode::Persistent ? c.ctas : 0u);
}

sph_status StepState::autotune(uint32_t trial_steps, bool allow_persistent, TuneChoice* out, bool* from_cache)
{
    if (trial_steps == 0 || tiles.empty()) {
        set_last_error("autotune: no steps or no particles");
        return SPH_ERR_INVALID_ARGUMENT;
    }
    const std::string key = tune_key(allow_persistent);
    {
        std::lock_guard<std::mutex> lock(g_tune_mutex);
        load_cache_file();
        auto it = g_tune_cache.find(key);
        if (it != g_tune_cache.end()) {
            apply_choice(it->second);
            *out = it->second;
            if (from_cache) *from_cache = true;
            return SPH_OK;
        }
    }
    if (from_cache) *from_cache = false;
    uint32_t sms = 0, per_sm = 0;
    sph_status st = persistent_capacity(&sms, &per_sm);
    if (st != SPH_OK) return st;
    if ((st = save_state()) != SPH_OK) return st;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    CUDA_TRY(cudaEventCreate(&e0));
    CUDA_TRY(cudaEventCreate(&e1));
    auto trial = [&](TuneChoice& c) -> sph_status {
        apply_choice(c);
        // one untimed step (graph capture, first-launch costs), then timed steps
        sph_status s = enqueue_steps(1, c.mode, false, false);
        if (s != SPH_OK) return s;
        CUDA_TRY(cudaEventRecord(e0, stream_));
        if ((s = enqueue_steps(trial_steps, c.mode, false, false)) != SPH_OK) return s;
        CUDA_TRY(cudaEventRecord(e1, stream_));
        CUDA_TRY(cudaEventSynchronize(e1));
        CUDA_TRY(cudaEventElapsedTime(&c.ms, e0, e1));
        c.ms /= (float)trial_steps;
        if ((s = check_device_error()) != SPH_OK) return s;
        return restore_state();
    };
    TuneChoice best{StepMode::Staged, 0u, 0, 0, 0.f};
    sph_status result = trial(best);
    const int shapes = exact_ ? 1 : kShapeCount;     // the exact passes have one shape
    const int force_shapes = exact_ ? 1 : kForceShapeCount;
    for (int d = 1; result == SPH_OK && d < shapes; ++d) {
        TuneChoice c{StepMode::Staged, 0u, d, 0, 0.f};
        if ((result = trial(c)) == SPH_OK && c.ms < best.ms) best = c;
    }
    const int best_d = best.density_shape;
    for (int f = 1; result == SPH_OK && f < force_shapes; ++f) {
        TuneChoice c{StepMode::Staged, 0u, best_d, f, 0.f};
        if ((result = trial(c)) == SPH_OK && c.ms < best.ms) best = c;
    }
    for (uint32_t k = 1; result == SPH_OK && allow_persistent && k <= per_sm; ++k) {
        TuneChoice c{StepMode::Persistent, k * sms, 0, 0, 0.f};
        if ((result = trial(c)) == SPH_OK && c.ms < best.ms) best = c;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (result != SPH_OK) {
        restore_state();
        apply_choice(TuneChoice{StepMode::Staged, 0u, 0, 0, 0.f});
        return result;
    }
    apply_choice(best);
    *out = best;
    std::lock_guard<std::mutex> lock(g_tune_mutex);
    if (g_tune_cache.emplace(key, best).second) append_cache_file(key, best);
    return SPH_OK;
}

}  // namespace sph
