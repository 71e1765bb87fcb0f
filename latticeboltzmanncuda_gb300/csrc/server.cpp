// Continuous-batching solve server (lbm_server_*): a request loop that admits D2Q9 solve requests
// as device memory and slots free up and advances every admitted solve together, round by round,
// in one lbm_batch.
//
//   arrivals  requests carry an arrival time (seconds after the start of the run); the loop runs in
//             real time and moves each request to the wait queue when its time has come
//   admission first come, first served: the head of the queue is admitted when its slot's device
//             bytes fit into the budget next to the live solves (and a slot is free); a request that
//             is larger than the whole budget is rejected (LBM_ERR_BUDGET), an invalid one fails
//             alone (its own status) without stopping the others
//   rounds    every round is one launch per step for all live solves, min(round_steps, largest
//             remaining step count) steps long; each solve carries its remaining step count as the
//             batch slot's step budget, so one that finishes mid-round just stops there (its blocks
//             exit at once); requests that arrive meanwhile join at the next round boundary, so
//             their work overlaps on the device with the running ones
//   retire    the step counts are known on the host, so a solve that finishes in a round is retired
//             as soon as that round is queued: the read-back of its density and velocity is queued
//             behind the round (a batch ticket) and its slot freed, stream-ordered; the request
//             completes when the host has collected the ticket into its buffers
//   pipeline  batch work is only queued, never waited for, except that the loop keeps at most one
//             round queued ahead of the one running: after queuing round r it waits for round
//             r - 1, so admission, table rebuilds and retirement of round r + 1 are prepared on the
//             host while the device runs round r
//
// States stay on the device from admission to completion.  A wall-clock limit (time_limit) bounds
// the whole run: requests not finished by then end with LBM_ERR_TIMEOUT.
#include <algorithm>
#include <chrono>
#include <cstring>
#include <deque>
#include <string>
#include <thread>
#include <vector>

#include <cuda_runtime_api.h>
#include <nvtx3/nvToolsExt.h>

#include "lbm_capi.h"

namespace lbm {
lbm_status set_thread_error(lbm_status s, const std::string &msg);
}

struct lbm_server {
    lbm_server_config cfg{};
    lbm_batch *batch = nullptr;
    std::string err;
};

namespace {

using Clock = std::chrono::steady_clock;

double seconds_since(Clock::time_point t0) {
    return std::chrono::duration<double>(Clock::now() - t0).count();
}

struct Live {
    int64_t req;
    int32_t slot;
    int64_t remaining;
    int64_t bytes;
};

}  // namespace

extern "C" {

LBM_API void lbm_server_config_init(lbm_server_config *c) {
    if (!c) return;
    std::memset(c, 0, sizeof(*c));
    c->dtype = LBM_F32;
    c->budget_bytes = (int64_t)150 * 1000 * 1000 * 1000;
    c->max_slots = 0;
    c->round_steps = 200;
    c->time_limit = 0.0;
}

LBM_API lbm_status lbm_server_create(const lbm_server_config *cfg, lbm_server **out) {
    if (!cfg || !out) return lbm::set_thread_error(LBM_ERR_INVALID, "lbm_server_create: null argument");
    *out = nullptr;
    if (cfg->budget_bytes <= 0 || cfg->round_steps < 1 || cfg->max_slots < 0 || cfg->time_limit < 0)
        return lbm::set_thread_error(LBM_ERR_INVALID, "lbm_server_create: bad configuration");
    lbm_server *s = new lbm_server();
    s->cfg = *cfg;
    lbm_status st = lbm_batch_create(cfg->dtype, cfg->device, cfg->stream, &s->batch);
    if (st != LBM_OK) {
        delete s;
        return st;
    }
    *out = s;
    return LBM_OK;
}

LBM_API lbm_status lbm_server_destroy(lbm_server *s) {
    if (!s) return LBM_OK;
    lbm_batch_destroy(s->batch);
    delete s;
    return LBM_OK;
}

LBM_API const char *lbm_server_last_error(const lbm_server *s) { return s ? s->err.c_str() : ""; }

LBM_API lbm_status lbm_server_run(lbm_server *s, const lbm_request *reqs, int64_t n, lbm_request_result *results,
                                  lbm_server_stats *stats) {
    nvtxRangePushA("lbm_server_run");
    struct PopRange {
        ~PopRange() { nvtxRangePop(); }
    } pop_range;
    if (!s || (n > 0 && (!reqs || !results)))
        return lbm::set_thread_error(LBM_ERR_INVALID, "lbm_server_run: null argument");
    const lbm_server_config &cfg = s->cfg;
    std::vector<int64_t> order((size_t)n);
    for (int64_t i = 0; i < n; ++i) order[(size_t)i] = i;
    std::stable_sort(order.begin(), order.end(), [&](int64_t a, int64_t b) { return reqs[a].arrival < reqs[b].arrival; });
    for (int64_t i = 0; i < n; ++i) {
        results[i].admitted = -1.0;
        results[i].finished = -1.0;
        results[i].status = LBM_ERR_STATE;
        results[i].slot = -1;
    }
    lbm_server_stats st{};
    std::deque<int64_t> waiting;
    std::vector<Live> live;
    size_t next = 0;
    int64_t done = 0, used = 0;
    lbm_status run_status = LBM_OK;
    const Clock::time_point t0 = Clock::now();

    struct Retiring {
        int64_t req, ticket;
    };
    std::deque<Retiring> retiring;
    cudaStream_t stream = nullptr;
    // per round: an event before its launch sequence and one after (timed: device seconds of the
    // rounds), two rounds in flight
    cudaEvent_t round_start[2] = {nullptr, nullptr}, round_done[2] = {nullptr, nullptr};
    bool events_ok = lbm_batch_get_stream(s->batch, reinterpret_cast<void **>(&stream)) == LBM_OK;
    for (int k = 0; k < 2 && events_ok; ++k)
        events_ok = cudaEventCreate(&round_start[k]) == cudaSuccess && cudaEventCreate(&round_done[k]) == cudaSuccess;
    auto destroy_events = [&]() {
        for (int k = 0; k < 2; ++k) {
            if (round_start[k]) cudaEventDestroy(round_start[k]);
            if (round_done[k]) cudaEventDestroy(round_done[k]);
        }
    };
    if (!events_ok) {
        destroy_events();
        cudaGetLastError();
        return lbm::set_thread_error(LBM_ERR_CUDA, "lbm_server_run: round events");
    }

    auto finish = [&](int64_t r, int32_t status) {
        results[r].status = status;
        results[r].finished = seconds_since(t0);
        ++done;
    };
    // collect the read-backs that have landed (all of them, waiting, with wait_all)
    auto collect = [&](bool wait_all) -> lbm_status {
        while (!retiring.empty()) {
            const Retiring rt = retiring.front();
            const lbm_request &q = reqs[rt.req];
            int32_t ready = 0;
            const lbm_status c = lbm_batch_collect(s->batch, rt.ticket, wait_all ? 1 : 0, q.out_rho, q.out_ux, q.out_uy, &ready);
            if (c != LBM_OK) {
                retiring.pop_front();
                finish(rt.req, c);
                return c;
            }
            if (!ready) break;  // tickets complete in queue order
            retiring.pop_front();
            finish(rt.req, LBM_OK);
        }
        return LBM_OK;
    };

    int64_t round = 0;
    while (done < n) {
        double now = seconds_since(t0);
        if (cfg.time_limit > 0 && now > cfg.time_limit) {
            run_status = LBM_ERR_TIMEOUT;
            break;
        }
        while (next < order.size() && reqs[order[next]].arrival <= now) waiting.push_back(order[next++]);

        // admission, first come first served (queued behind the running round)
        while (!waiting.empty()) {
            const int64_t r = waiting.front();
            const lbm_request &q = reqs[r];
            const int64_t bytes = lbm_batch_slot_bytes(cfg.dtype, q.nx, q.ny);
            if (bytes < 0 || q.steps < 0) {
                waiting.pop_front();
                results[r].admitted = seconds_since(t0);
                finish(r, LBM_ERR_INVALID);
                continue;
            }
            if (bytes > cfg.budget_bytes) {
                waiting.pop_front();
                results[r].admitted = seconds_since(t0);
                finish(r, LBM_ERR_BUDGET);
                ++st.rejected;
                continue;
            }
            if (used + bytes > cfg.budget_bytes) break;
            if (cfg.max_slots > 0 && (int64_t)live.size() >= cfg.max_slots) break;
            lbm_desc d;
            lbm_desc_init(&d);
            d.mode = LBM_D2Q9;
            d.nx = q.nx;
            d.ny = q.ny;
            d.nz = 1;
            d.tau = q.tau;
            d.periodic = q.periodic;
            d.body_force[0] = q.body_force[0];
            d.body_force[1] = q.body_force[1];
            d.wall_velocity[0] = q.wall_velocity[0];
            d.wall_velocity[1] = q.wall_velocity[1];
            int32_t slot = -1;
            const lbm_status a = lbm_batch_add(s->batch, &d, q.flags, &slot);
            waiting.pop_front();
            results[r].admitted = seconds_since(t0);
            if (a == LBM_ERR_OOM) {
                // the device had less room than the budget promised: fail this request, keep serving
                finish(r, LBM_ERR_OOM);
                continue;
            }
            if (a != LBM_OK) {
                finish(r, a);
                continue;
            }
            results[r].slot = slot;
            lbm_batch_set_slot_steps(s->batch, slot, q.steps);
            used += bytes;
            live.push_back(Live{r, slot, q.steps, bytes});
            st.peak_bytes = std::max(st.peak_bytes, used);
            st.peak_slots = std::max<int32_t>(st.peak_slots, (int32_t)live.size());
        }

        if (live.empty()) {
            if (!retiring.empty()) {  // nothing to queue: wait for the read-backs in flight
                if ((run_status = collect(true)) != LBM_OK) break;
                continue;
            }
            if (next < order.size()) {
                // idle until the next arrival (bounded sleeps; the time limit is checked each pass)
                const double wait = reqs[order[next]].arrival - seconds_since(t0);
                if (wait > 0) std::this_thread::sleep_for(std::chrono::duration<double>(std::min(wait, 0.01)));
                continue;
            }
            if (waiting.empty()) break;
            continue;
        }

        int64_t longest = 0;
        for (const Live &l : live) longest = std::max(longest, l.remaining);
        const int64_t k = std::min<int64_t>(cfg.round_steps, longest);
        lbm_status e = cudaEventRecord(round_start[round & 1], stream) == cudaSuccess ? LBM_OK : LBM_ERR_CUDA;
        if (e == LBM_OK && k > 0) e = lbm_batch_step(s->batch, (int32_t)k);
        if (e == LBM_OK && cudaEventRecord(round_done[round & 1], stream) != cudaSuccess) e = LBM_ERR_CUDA;
        if (e != LBM_OK) {
            s->err = lbm_batch_last_error(s->batch);
            run_status = e;
            break;
        }
        ++st.rounds;
        // retire the solves this round finishes: read-back and free queued behind it
        std::vector<Live> still;
        still.reserve(live.size());
        for (Live &l : live) {
            const int64_t adv = std::min(k, l.remaining);
            l.remaining -= adv;
            st.cell_updates += (double)reqs[l.req].nx * reqs[l.req].ny * (double)adv;
            if (l.remaining > 0) {
                still.push_back(l);
                continue;
            }
            int64_t ticket = 0;
            const lbm_status o = lbm_batch_moments_async(s->batch, l.slot, &ticket);
            lbm_batch_remove(s->batch, l.slot);
            used -= l.bytes;
            if (o != LBM_OK)
                finish(l.req, o);
            else
                retiring.push_back(Retiring{l.req, ticket});
        }
        live.swap(still);
        // at most one round queued ahead of the running one
        if (round > 0) {
            const int p = (int)((round - 1) & 1);
            float ms = 0.0f;
            if (cudaEventSynchronize(round_done[p]) != cudaSuccess ||
                cudaEventElapsedTime(&ms, round_start[p], round_done[p]) != cudaSuccess) {
                cudaGetLastError();
                s->err = "lbm_server_run: a round failed on the device";
                run_status = LBM_ERR_CUDA;
                break;
            }
            st.round_seconds += ms * 1e-3;
        }
        ++round;
        if ((run_status = collect(false)) != LBM_OK) break;
    }
    if (run_status == LBM_OK && round > 0) {  // the last round's device time
        const int p = (int)((round - 1) & 1);
        float ms = 0.0f;
        if (cudaEventSynchronize(round_done[p]) == cudaSuccess &&
            cudaEventElapsedTime(&ms, round_start[p], round_done[p]) == cudaSuccess)
            st.round_seconds += ms * 1e-3;
        cudaGetLastError();
    }
    if (run_status == LBM_OK) run_status = collect(true);
    else lbm_batch_synchronize(s->batch);
    {
        int64_t info[8];
        if (lbm_batch_info(s->batch, info) == LBM_OK) {
            st.tile_shape[0] = (int32_t)info[4];
            st.tile_shape[1] = (int32_t)info[5];
            st.tile_shape[2] = (int32_t)info[6];
        }
        lbm_batch_tunings(s->batch, &st.tunings);
    }

    // anything left ends with the run's status (time limit or a device error)
    for (const Live &l : live) {
        lbm_batch_remove(s->batch, l.slot);
        if (results[l.req].finished < 0) finish(l.req, run_status == LBM_OK ? LBM_ERR_STATE : run_status);
    }
    for (int64_t r : waiting)
        if (results[r].finished < 0) finish(r, run_status == LBM_OK ? LBM_ERR_STATE : run_status);
    for (; next < order.size(); ++next)
        if (results[order[next]].finished < 0) finish(order[next], run_status == LBM_OK ? LBM_ERR_STATE : run_status);
    for (const Retiring &rt : retiring)
        if (results[rt.req].finished < 0) finish(rt.req, run_status == LBM_OK ? LBM_ERR_STATE : run_status);
    destroy_events();
    st.makespan = seconds_since(t0);
    if (stats) *stats = st;
    if (run_status != LBM_OK) {
        s->err = s->err.empty() ? std::string("lbm_server_run: ") + lbm_status_string(run_status) : s->err;
        return lbm::set_thread_error(run_status, s->err);
    }
    return LBM_OK;
}

}  // extern "C"
