// sph_server.cu -- continuous batching of simulation jobs on one GPU.
//
// The reference has no serving layer (it advances one scene per engine,
// SimulationEngineCPU.cpp:420-459); this is the served form of the same step.
// Jobs wait in a FIFO queue.  A job is admitted when its resident bytes fit
// the HBM budget and a slot is free (queued jobs behind a job that does not
// fit may pass it).  An admitted job is uploaded into its own ranges of one
// device arena and sorted alone, so admissions and retirements never move
// another job's state.  Every poll advances all admitted jobs together with
// the staged step (its CUDA graph of stage kernels, rebuilt when the scene
// table changes) over the current scene table, by the smallest number of
// steps any of them still needs (at most chunk_steps),
// so each job stops exactly at its horizon; finished jobs are read back and
// their ranges freed.  Polls are pipelined with the GPU: a poll queues its
// steps and returns, and the next one waits for them, retires the jobs they
// finished and queues the next round.  On GB300 the kernels read a job's
// particles from the caller's host arrays and write its results into host
// memory directly (Grace's address translation), so no host copy or wait
// sits between rounds.
#include <algorithm>
#include <chrono>
#include <deque>
#include <map>
#include <memory>
#include <new>
#include <unordered_map>

#include "sph_state.h"

using sph::SceneDesc;
using sph::SceneInput;
using sph::StepState;

namespace {

constexpr uint64_t kAlign = 32;   // range starts: 128-byte aligned bucket tables

// First-fit allocator over an index space [0, cap).
class RangeAlloc {
public:
    void reset(uint64_t cap)
    {
        free_.clear();
        cap_ = cap;
        if (cap) free_[0] = cap;
    }
    uint64_t cap() const { return cap_; }
    // Extends the space to new_cap (the tail becomes free).
    void grow(uint64_t new_cap)
    {
        if (new_cap <= cap_) return;
        uint64_t start = cap_, len = new_cap - cap_;
        auto it = free_.lower_bound(start);
        if (it != free_.begin()) {
            auto prev = std::prev(it);
            if (prev->first + prev->second == start) {
                start = prev->first;
                len += prev->second;
                free_.erase(prev);
            }
        }
        free_[start] = len;
        cap_ = new_cap;
    }
    bool alloc(uint64_t len, uint64_t* off)
    {
        len = round(len);
        for (auto it = free_.begin(); it != free_.end(); ++it) {
            if (it->second >= len) {
                *off = it->first;
                const uint64_t rest = it->second - len;
                const uint64_t at = it->first + len;
                free_.erase(it);
                if (rest) free_[at] = rest;
                return true;
            }
        }
        return false;
    }
    void release(uint64_t off, uint64_t len)
    {
        len = round(len);
        auto it = free_.emplace(off, len).first;
        auto next = std::next(it);
        if (next != free_.end() && it->first + it->second == next->first) {
            it->second += next->second;
            free_.erase(next);
        }
        if (it != free_.begin()) {
            auto prev = std::prev(it);
            if (prev->first + prev->second == it->first) {
                prev->second += it->second;
                free_.erase(it);
            }
        }
    }
    // Smallest capacity that would fit `len` more at the tail.
    uint64_t needed_for(uint64_t len) const
    {
        len = round(len);
        uint64_t tail_free = 0;
        if (!free_.empty()) {
            auto last = std::prev(free_.end());
            if (last->first + last->second == cap_) tail_free = last->second;
        }
        return cap_ + (len > tail_free ? len - tail_free : 0);
    }
    static uint64_t round(uint64_t len) { return (std::max<uint64_t>(len, 1) + kAlign - 1) / kAlign * kAlign; }

private:
    std::map<uint64_t, uint64_t> free_;
    uint64_t cap_ = 0;
};

enum class JobState { Queued, Active, Finished };

struct Job {
    uint64_t id = 0;
    SceneInput in;
    std::vector<float> pos, spos;
    uint32_t steps = 0, done = 0;
    JobState state = JobState::Queued;
    uint64_t p_off = 0, q_off = 0, s_off = 0, sq_off = 0, sf_off = 0, sb_off = 0;
    uint64_t bytes = 0;
    std::vector<sph_dynamic_particle> result;
    cudaEvent_t ready = nullptr;     // the readback into `result` is complete when this fires
    float gas = 1.f, rho0 = 0.f;
};

double now_s()
{
    using namespace std::chrono;
    return duration<double>(steady_clock::now().time_since_epoch()).count();
}

}  // namespace

uint64_t job_bytes(uint32_t n, uint32_t s)
{
    // per dynamic particle: sorted pos/vel 32, unsorted pos/vel 32, staging 32,
    // key/arrival/ptag 12, buffer tags 8, two buckets x (count + start) 16,
    // neighbour lists (96 + 48 slots) 576, list counts 4;
    // per static particle: two sorted copies 32, staging 32, bucket count +
    // start for both tables 8 + 8 x 8 = 72
    // plus 8 bytes per static particle of static-presence bitmap
    return 712ull * n + 144ull * s + 4096ull;
}

struct sph_server {
    int device = 0;
    cudaStream_t stream = nullptr;
    uint64_t budget = 0;
    uint32_t max_slots = 0;
    StepState arena;
    bool arena_ready = false;
    RangeAlloc pa, qa, sa, sqa, sfa, sba;
    uint64_t used_bytes = 0;
    uint64_t next_id = 1;
    std::unordered_map<uint64_t, std::unique_ptr<Job>> jobs;
    std::deque<uint64_t> queue;
    std::vector<uint64_t> active;
    std::deque<uint64_t> finished;   // retired since the last sph_server_finished
    bool dirty = false;
    sph::StepMode mode = sph::StepMode::Staged;
    // host wall time per poll phase (sph_server_stats): admission (uploads
    // and sort launches), waiting for the admissions' sorts, rebuilding the
    // scene table, queueing the steps, waiting for them, reading back
    double phase_s[6] = {};
    uint64_t polls = 0, steps_run = 0, table_builds = 0;
    // the GPU reads job inputs and writes results in pageable host memory
    // itself (GB300: Grace's address translation), so admissions and
    // readbacks are queued without host copies or waits
    bool host_direct = false;
    // steps queued by the last poll, not yet waited for
    bool pending = false;
    uint32_t pending_steps = 0;
    cudaEvent_t steps_done = nullptr;
};

#define SRV_CUDA_TRY(expr)                                                                     \
    do {                                                                                       \
        cudaError_t e_ = (expr);                                                               \
        if (e_ != cudaSuccess) {                                                               \
            sph::set_last_error(std::string(#expr) + ": " + cudaGetErrorString(e_));           \
            return e_ == cudaErrorMemoryAllocation ? SPH_ERR_OUT_OF_MEMORY : SPH_ERR_CUDA;     \
        }                                                                                      \
    } while (0)

#define SRV_TRY(expr)                 \
    do {                              \
        sph_status s_ = (expr);       \
        if (s_ != SPH_OK) return s_;  \
    } while (0)

// Makes room in the arena for a job of n dynamic and s static particles.
static sph_status ensure_room(sph_server* sv, const Job& j)
{
    const uint64_t n = j.in.n, s = j.in.s, q = 2ull * j.in.n + 1, sq = (uint64_t)j.in.s + 1;
    const uint64_t sf = (uint64_t)sph::fast_static_buckets(j.in.s) + 1;
    const uint64_t sb = sph::static_bitmap_bits(j.in.s) / 32 + 1;
    uint64_t need_n = sv->pa.needed_for(n), need_q = sv->qa.needed_for(q);
    uint64_t need_s = sv->sa.needed_for(s), need_sq = sv->sqa.needed_for(sq), need_sf = sv->sfa.needed_for(sf);
    uint64_t need_sb = sv->sba.needed_for(sb);
    if (need_n <= sv->pa.cap() && need_q <= sv->qa.cap() && need_s <= sv->sa.cap() && need_sq <= sv->sqa.cap() &&
        need_sf <= sv->sfa.cap() && need_sb <= sv->sba.cap())
        return SPH_OK;
    auto grown = [](uint64_t need, uint64_t cap) { return need <= cap ? cap : std::max(need, cap * 2); };
    uint64_t cn = grown(need_n, sv->pa.cap()), cq = grown(need_q, sv->qa.cap());
    uint64_t cs = grown(need_s, sv->sa.cap()), csq = grown(need_sq, sv->sqa.cap());
    uint64_t csf = grown(need_sf, sv->sfa.cap()), csb = grown(need_sb, sv->sba.cap());
    const uint64_t limit = (1ull << 31) - 64;
    if (cn > limit || cq > limit || cs > limit || csq > limit || csf > limit || csb > limit) {
        sph::set_last_error("arena index space exhausted");
        return SPH_ERR_CAPACITY;
    }
    if (!sv->arena_ready) {
        SRV_TRY(sv->arena.init_arena(sv->device, sv->stream, (uint32_t)cn, (uint32_t)cq, (uint32_t)cs, (uint32_t)csq,
                                     (uint32_t)csf, (uint32_t)csb, sv->max_slots));
        sv->arena_ready = true;
    } else {
        SRV_TRY(sv->arena.grow_arena((uint32_t)cn, (uint32_t)cq, (uint32_t)cs, (uint32_t)csq, (uint32_t)csf,
                                     (uint32_t)csb));
    }
    sv->pa.grow(cn);
    sv->qa.grow(cq);
    sv->sa.grow(cs);
    sv->sqa.grow(csq);
    sv->sfa.grow(csf);
    sv->sba.grow(csb);
    return SPH_OK;
}

static SceneDesc desc_of(const Job& j)
{
    SceneDesc d = sph::scene_desc_for(j.in);
    d.p_off = (uint32_t)j.p_off;
    d.q_off = (uint32_t)j.q_off;
    d.s_off = (uint32_t)j.s_off;
    d.sq_off = (uint32_t)j.sq_off;
    d.sf_off = (uint32_t)j.sf_off;
    d.sbm_off = (uint32_t)j.sb_off;
    return d;
}

static sph_status admit(sph_server* sv, Job& j)
{
    SRV_TRY(ensure_room(sv, j));
    const uint64_t n = j.in.n, q = 2ull * j.in.n + 1, s = j.in.s, sq = (uint64_t)j.in.s + 1;
    const uint64_t sf = (uint64_t)sph::fast_static_buckets(j.in.s) + 1;
    bool ok = sv->pa.alloc(n, &j.p_off);
    ok = ok && sv->qa.alloc(q, &j.q_off);
    ok = ok && sv->sa.alloc(s, &j.s_off);
    ok = ok && sv->sqa.alloc(sq, &j.sq_off);
    ok = ok && sv->sfa.alloc(sf, &j.sf_off);
    ok = ok && sv->sba.alloc(sph::static_bitmap_bits(j.in.s) / 32 + 1, &j.sb_off);
    if (!ok) {
        sph::set_last_error("arena allocation failed after growth");
        return SPH_ERR_CAPACITY;
    }
    SceneInput in = j.in;
    in.pos = j.pos.data();
    in.spos = j.spos.empty() ? nullptr : j.spos.data();
    SRV_TRY(sv->arena.admit_scene(desc_of(j), in, /*sync=*/false, sv->host_direct));
    if (!sv->host_direct) {    // the inputs were copied; kernels read them in place otherwise
        j.pos.clear();
        j.pos.shrink_to_fit();
        j.spos.clear();
        j.spos.shrink_to_fit();
    }
    j.state = JobState::Active;
    sv->used_bytes += j.bytes;
    sv->active.push_back(j.id);
    sv->dirty = true;
    return SPH_OK;
}

static void release_ranges(sph_server* sv, Job& j)
{
    sv->pa.release(j.p_off, j.in.n);
    sv->qa.release(j.q_off, 2ull * j.in.n + 1);
    sv->sa.release(j.s_off, j.in.s);
    sv->sqa.release(j.sq_off, (uint64_t)j.in.s + 1);
    sv->sfa.release(j.sf_off, (uint64_t)sph::fast_static_buckets(j.in.s) + 1);
    sv->sba.release(j.sb_off, sph::static_bitmap_bits(j.in.s) / 32 + 1);
    sv->used_bytes -= j.bytes;
}

extern "C" {

SPH_API uint64_t sph_server_job_bytes(uint32_t n, uint32_t s) { return job_bytes(n, s); }

SPH_API sph_status sph_server_create(sph_server** out, int device, uint64_t hbm_budget_bytes, uint32_t max_slots)
{
    if (!out || hbm_budget_bytes == 0 || max_slots == 0) return SPH_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    int count = 0;
    SRV_CUDA_TRY(cudaGetDeviceCount(&count));
    if (device < 0 || device >= count) {
        sph::set_last_error("no such CUDA device");
        return SPH_ERR_INVALID_ARGUMENT;
    }
    SRV_CUDA_TRY(cudaSetDevice(device));
    sph_server* sv = new (std::nothrow) sph_server();
    if (!sv) return SPH_ERR_OUT_OF_MEMORY;
    cudaError_t e = cudaStreamCreateWithFlags(&sv->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        delete sv;
        sph::set_last_error(cudaGetErrorString(e));
        return SPH_ERR_CUDA;
    }
    sv->device = device;
    sv->budget = hbm_budget_bytes;
    sv->max_slots = max_slots;
    int pageable = 0;
    if (cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, device) == cudaSuccess)
        sv->host_direct = pageable != 0;
    e = cudaEventCreateWithFlags(&sv->steps_done, cudaEventDisableTiming);
    if (e != cudaSuccess) {
        cudaStreamDestroy(sv->stream);
        delete sv;
        sph::set_last_error(cudaGetErrorString(e));
        return SPH_ERR_CUDA;
    }
    *out = sv;
    return SPH_OK;
}

SPH_API sph_status sph_server_destroy(sph_server* sv)
{
    if (!sv) return SPH_ERR_INVALID_ARGUMENT;
    cudaSetDevice(sv->device);
    cudaStreamSynchronize(sv->stream);
    for (auto& kv : sv->jobs)
        if (kv.second->ready) cudaEventDestroy(kv.second->ready);
    sv->arena.release();
    cudaEventDestroy(sv->steps_done);
    cudaStreamDestroy(sv->stream);
    delete sv;
    return SPH_OK;
}

SPH_API sph_status sph_server_submit(sph_server* sv, const sph_params* params, const float* dyn_pos, uint32_t n,
                                     const float* static_pos, uint32_t s, float dt, uint32_t steps, uint64_t* job_id)
{
    if (!sv || !params || !job_id) return SPH_ERR_INVALID_ARGUMENT;
    if (n == 0 || steps == 0 || !(dt > 0.f)) {
        sph::set_last_error("a job needs particles, a positive dt and at least one step");
        return SPH_ERR_INVALID_ARGUMENT;
    }
    SceneInput in;
    in.params = *params;
    in.n = n;
    in.s = s;
    in.dt = dt;
    in.pos = dyn_pos;
    in.spos = static_pos;
    SRV_TRY(sph::validate_scene(in));
    auto j = std::make_unique<Job>();
    j->bytes = job_bytes(n, s);
    if (j->bytes > sv->budget) {
        sph::set_last_error("job alone exceeds the HBM budget");
        return SPH_ERR_BUDGET;
    }
    j->id = sv->next_id++;
    j->in = in;
    j->pos.assign(dyn_pos, dyn_pos + 3ull * n);
    if (s) j->spos.assign(static_pos, static_pos + 3ull * s);
    j->in.pos = nullptr;
    j->in.spos = nullptr;
    j->steps = steps;
    j->gas = params->gas_constant;
    j->rho0 = params->rest_density;
    *job_id = j->id;
    sv->queue.push_back(j->id);
    sv->jobs.emplace(j->id, std::move(j));
    return SPH_OK;
}

SPH_API sph_status sph_server_set_exact(sph_server* sv, int exact)
{
    if (!sv) return SPH_ERR_INVALID_ARGUMENT;
    SRV_CUDA_TRY(cudaSetDevice(sv->device));
    SRV_CUDA_TRY(cudaStreamSynchronize(sv->stream));
    sv->arena.set_exact(exact != 0);
    return SPH_OK;
}

// One scheduling round, pipelined with the GPU: it waits for the steps the
// previous round queued, retires the jobs they finished (their readback is
// queued into host memory), admits queued jobs (uploads and sorts queued),
// rebuilds the scene table if it changed and queues this round's steps, then
// returns while the GPU runs them.  So the host's bookkeeping and the
// caller's work between rounds overlap the steps.
SPH_API sph_status sph_server_poll(sph_server* sv, uint32_t chunk_steps, uint32_t* active_out, uint32_t* queued_out)
{
    if (!sv || chunk_steps == 0) return SPH_ERR_INVALID_ARGUMENT;
    SRV_CUDA_TRY(cudaSetDevice(sv->device));
    double t = now_s();
    auto lap = [&](int phase) {
        const double t1 = now_s();
        sv->phase_s[phase] += t1 - t;
        t = t1;
    };
    ++sv->polls;
    if (sv->pending) {
        SRV_CUDA_TRY(cudaEventSynchronize(sv->steps_done));
        SRV_TRY(sv->arena.check_device_error());   // the round's admissions and steps
        lap(4);
        sv->pending = false;
        std::vector<uint64_t> still;
        for (size_t k = 0; k < sv->active.size(); ++k) {
            Job& j = *sv->jobs[sv->active[k]];
            j.done += sv->pending_steps;
            if (j.done < j.steps) {
                still.push_back(j.id);
                continue;
            }
            j.result.resize(j.in.n);
            if (sv->host_direct) {
                SRV_TRY(sv->arena.read_scene_async((uint32_t)k, j.result.data()));
                SRV_CUDA_TRY(cudaEventCreateWithFlags(&j.ready, cudaEventDisableTiming));
                SRV_CUDA_TRY(cudaEventRecord(j.ready, sv->stream));
            } else {
                SRV_TRY(sv->arena.read_scene((uint32_t)k, j.result.data(), nullptr));
            }
            j.state = JobState::Finished;
            release_ranges(sv, j);          // a range reused below is written after the readback
            sv->finished.push_back(j.id);
            sv->dirty = true;
        }
        sv->active.swap(still);
        lap(5);
    }
    // admit in arrival order; later jobs may pass one that does not fit
    for (auto it = sv->queue.begin(); it != sv->queue.end() && sv->active.size() < sv->max_slots;) {
        Job& j = *sv->jobs[*it];
        if (sv->used_bytes + j.bytes <= sv->budget) {
            SRV_TRY(admit(sv, j));
            it = sv->queue.erase(it);
        } else {
            ++it;
        }
    }
    lap(0);
    if (!sv->active.empty()) {
        if (sv->dirty) {
            std::vector<SceneDesc> descs;
            for (uint64_t id : sv->active) descs.push_back(desc_of(*sv->jobs[id]));
            SRV_TRY(sv->arena.set_active(descs));
            sv->dirty = false;
            ++sv->table_builds;
        }
        lap(2);
        uint32_t steps = chunk_steps;
        for (uint64_t id : sv->active) {
            const Job& j = *sv->jobs[id];
            steps = std::min(steps, j.steps - j.done);
        }
        SRV_TRY(sv->arena.enqueue_steps(steps, sv->mode, false, false));
        SRV_CUDA_TRY(cudaEventRecord(sv->steps_done, sv->stream));
        sv->pending = true;
        sv->pending_steps = steps;
        sv->steps_run += steps;
        lap(3);
    }
    if (active_out) *active_out = (uint32_t)sv->active.size();
    if (queued_out) *queued_out = (uint32_t)sv->queue.size();
    return SPH_OK;
}

SPH_API sph_status sph_server_stats(sph_server* sv, double* phase_seconds, uint64_t* counts)
{
    if (!sv) return SPH_ERR_INVALID_ARGUMENT;
    if (phase_seconds)
        for (int k = 0; k < 6; ++k) phase_seconds[k] = sv->phase_s[k];
    if (counts) {
        counts[0] = sv->polls;
        counts[1] = sv->steps_run;
        counts[2] = sv->table_builds;
    }
    return SPH_OK;
}

SPH_API sph_status sph_server_finished(sph_server* sv, uint64_t* job_ids, uint32_t capacity, uint32_t* count)
{
    if (!sv || !count || (capacity && !job_ids)) return SPH_ERR_INVALID_ARGUMENT;
    uint32_t k = 0;
    while (k < capacity && !sv->finished.empty()) {
        job_ids[k++] = sv->finished.front();
        sv->finished.pop_front();
    }
    *count = k;
    return SPH_OK;
}

SPH_API sph_status sph_server_result(sph_server* sv, uint64_t job_id, sph_dynamic_particle* out, float* density)
{
    if (!sv) return SPH_ERR_INVALID_ARGUMENT;
    auto it = sv->jobs.find(job_id);
    if (it == sv->jobs.end() || it->second->state != JobState::Finished) {
        sph::set_last_error("job unknown or not finished");
        return SPH_ERR_NOT_FOUND;
    }
    Job& j = *it->second;
    if (j.ready) {                       // a readback still in flight
        SRV_CUDA_TRY(cudaSetDevice(sv->device));
        SRV_CUDA_TRY(cudaEventSynchronize(j.ready));
        cudaEventDestroy(j.ready);
        j.ready = nullptr;
    }
    if (out) std::copy(j.result.begin(), j.result.end(), out);
    if (density)
        for (uint32_t i = 0; i < j.in.n; ++i) density[i] = j.result[i].pressure / j.gas + j.rho0;
    sv->jobs.erase(it);
    return SPH_OK;
}

}  // extern "C"
