// server.cpp -- continuous-batching solve server (no reference counterpart:
// the reference runs one case per process, src/main.cu:75-102).
//
// Requests (a METHOD-mode case and a step count) wait in FIFO order.  At each
// tick the waiting requests that fit in the device-memory budget are admitted
// together as one cohort: one batched solver on its own CUDA stream, state
// resident on the device until the request finishes.  Every live cohort then
// advances up to steps_per_tick time steps (never past the first of its
// requests to finish); the steps of all cohorts are issued before any is
// waited for, so cohorts admitted at different times overlap on the GPU.  A
// request that has done its steps is copied out (u, v, p, statistics) and
// made inactive in its cohort, which stops its work while the other members
// go on; a cohort whose members have all finished frees its memory, and the
// next tick admits more requests.  A request's result does not depend on the
// cohort it ran in: instances in a batch share no arithmetic.
//
// Pre-emption: a running request can be taken off the device between ticks.
// Its state is kept as a binary checkpoint in host memory (ifx_checkpoint_save),
// its instance is made inactive, and it waits again; when it is admitted
// again, its new instance loads the checkpoint and the request continues bit
// for bit.
#include <algorithm>
#include <cstring>
#include <deque>
#include <list>
#include <map>
#include <vector>

#include "ifx_host.h"

namespace ifx {

// Device bytes of one METHOD-mode instance (the allocations of create_method:
// 26 FP64 cell fields, cell types, ghost index map, two multigrid buffers and
// a residual per level in T plus stencil bytes), rounded up by 10% for the
// ghost tables, 1-D metrics and per-level tables.
size_t estimate_instance_bytes(const ifx_config& c) {
    const size_t nx = (size_t)c.nx + 2, ny = (size_t)c.ny + 2;
    const size_t pitch = (nx + 31) / 32 * 32;
    const size_t cells = pitch * ny;
    const size_t ts = c.precision == IFX_PREC_FP64 ? 8 : 4;
    const size_t per_cell = 26 * 8 + 1 + 4;
    const size_t levels = cells * 4 / 3 * (3 * ts + 1);
    return (cells * per_cell + levels) * 11 / 10 + (1u << 20);
}

}  // namespace ifx

using namespace ifx;

struct ifx_server {
    struct Request {
        long long id = 0;
        ifx_config cfg;
        std::vector<double> xf, yf;
        int nsteps = 0, done = 0;
        int state = 0;  // 0 waiting, 1 running, 2 finished, 3 failed
        size_t est = 0;
        int nx = 0, ny = 0;
        std::vector<double> u, v, p;
        ifx_stats st;
        std::vector<char> resume;  // checkpoint of a pre-empted request
    };
    struct Cohort {
        ifx_solver* s = nullptr;
        std::vector<long long> ids;  // per instance; -1 once its request was pre-empted
        int live = 0;
        int pending = 0;  // steps issued this tick
        size_t bytes = 0;
    };
    size_t budget = 0, used = 0;
    int max_cohort = 64;
    int steps_per_tick = 1;  // a cohort advances up to this many steps per tick
    int exec_mode = IFX_EXEC_GRAPH;
    int mg_rows = 0;                  // tile rows of the cohorts; 0: by precision and size
    long long wide_cells = 1 << 18;   // mixed cohorts from this many cells use four rows
    long long next_id = 1;
    std::map<long long, Request> reqs;
    std::deque<long long> waiting;
    std::deque<long long> finished;
    std::list<Cohort> cohorts;
};

static ifx_status admit(ifx_server* V) {
    std::vector<long long> take;
    size_t want = 0;
    while (!V->waiting.empty() && (int)take.size() < V->max_cohort) {
        ifx_server::Request& r = V->reqs[V->waiting.front()];
        if (r.est > V->budget) {  // can never fit
            r.state = 3;
            V->finished.push_back(r.id);
            V->waiting.pop_front();
            continue;
        }
        if (V->used + want + r.est > V->budget) break;
        // a batch shares its precision and multigrid sweep counts: the first
        // request that differs from the cohort's first one starts the next cohort
        if (!take.empty()) {
            const ifx_config& a = V->reqs[take[0]].cfg;
            if (r.cfg.precision != a.precision || r.cfg.mg_pre != a.mg_pre || r.cfg.mg_post != a.mg_post) break;
        }
        want += r.est;
        take.push_back(r.id);
        V->waiting.pop_front();
    }
    if (take.empty()) return IFX_OK;
    std::vector<ifx_config> cfgs;
    std::vector<const double*> xs, ys;
    for (long long id : take) {
        ifx_server::Request& r = V->reqs[id];
        cfgs.push_back(r.cfg);
        xs.push_back(r.xf.data());
        ys.push_back(r.yf.data());
    }
    ifx_server::Cohort c;
    ifx_status st = ifx_create_batch((int)take.size(), cfgs.data(), xs.data(), ys.data(), &c.s);
    if (st == IFX_OK && V->exec_mode != IFX_EXEC_DEFAULT) st = ifx_set_exec_mode(c.s, V->exec_mode);
    if (st == IFX_OK) {
        // multigrid and finest-level tile shape: four rows per thread for mixed
        // cohorts with many cells (the latency-bound phases then keep more loads
        // in flight), one row otherwise; results do not depend on it
        long long cells = 0;
        for (const ifx_config& c : cfgs) cells += (long long)c.nx * c.ny;
        int rows = V->mg_rows;
        if (rows == 0) rows = (cfgs[0].precision == IFX_PREC_MIXED && cells >= V->wide_cells) ? 4 : 1;
        st = ifx_set_mg_tile_rows(c.s, rows);
    }
    if (st != IFX_OK) {
        if (c.s) ifx_destroy(c.s);
        for (long long id : take) {
            V->reqs[id].state = 3;
            V->finished.push_back(id);
        }
        return st;
    }
    c.ids = take;
    c.live = (int)take.size();
    ifx_status worst = IFX_OK;
    for (size_t k = 0; k < take.size(); k++) {
        ifx_server::Request& r = V->reqs[take[k]];
        r.state = 1;
        ifx_get_dims(c.s, (int)k, &r.nx, &r.ny);
        if (!r.resume.empty()) {
            const ifx_status e = ifx_checkpoint_load(c.s, (int)k, r.resume.data(), r.resume.size());
            if (e != IFX_OK) {
                ifx_set_instance_active(c.s, (int)k, 0);
                r.state = 3;
                V->finished.push_back(r.id);
                c.live--;
                worst = e;
            }
            r.resume.clear();
            r.resume.shrink_to_fit();
        }
    }
    ifx_device_bytes(c.s, &c.bytes);
    V->used += c.bytes;
    V->cohorts.push_back(c);
    return worst;
}

extern "C" ifx_status ifx_estimate_bytes(const ifx_config* cfg, size_t* bytes) {
    if (!cfg || !bytes) return set_error(IFX_ERR_ARG, "ifx_estimate_bytes: bad argument");
    *bytes = estimate_instance_bytes(*cfg);
    return IFX_OK;
}

extern "C" ifx_status ifx_server_create(size_t hbm_budget_bytes, int max_cohort, ifx_server** out) {
    if (!out || hbm_budget_bytes == 0 || max_cohort < 1) return set_error(IFX_ERR_ARG, "ifx_server_create: bad argument");
    ifx_server* V = new ifx_server();
    V->budget = hbm_budget_bytes;
    V->max_cohort = max_cohort;
    *out = V;
    return IFX_OK;
}

extern "C" ifx_status ifx_server_set_steps_per_tick(ifx_server* V, int steps) {
    if (!V || steps < 1) return set_error(IFX_ERR_ARG, "ifx_server_set_steps_per_tick: bad argument");
    V->steps_per_tick = steps;
    return IFX_OK;
}

extern "C" ifx_status ifx_server_set_exec_mode(ifx_server* V, int mode) {
    if (!V || mode < IFX_EXEC_DEFAULT || mode > IFX_EXEC_HOST) return set_error(IFX_ERR_ARG, "ifx_server_set_exec_mode: bad argument");
    V->exec_mode = mode;
    return IFX_OK;
}

extern "C" ifx_status ifx_server_submit(ifx_server* V, const ifx_config* cfg, const double* xf, const double* yf,
                                        int nsteps, long long* id) {
    if (!V || !cfg || !xf || !yf || nsteps < 1 || !id) return set_error(IFX_ERR_ARG, "ifx_server_submit: bad argument");
    if (cfg->mode != IFX_MODE_METHOD) return set_error(IFX_ERR_ARG, "ifx_server_submit: METHOD-mode cases only");
    {   // refused here rather than failing the cohort it would be admitted with
        const ifx_status st = validate_method_config(cfg);
        if (st != IFX_OK) return st;
    }
    ifx_server::Request r;
    r.id = V->next_id++;
    r.cfg = *cfg;
    r.xf.assign(xf, xf + cfg->nx + 1);
    r.yf.assign(yf, yf + cfg->ny + 1);
    r.nsteps = nsteps;
    r.est = estimate_instance_bytes(*cfg);
    std::memset(&r.st, 0, sizeof(r.st));
    *id = r.id;
    V->reqs[r.id] = std::move(r);
    V->waiting.push_back(*id);
    return IFX_OK;
}

extern "C" ifx_status ifx_server_tick(ifx_server* V, int* n_finished) {
    if (!V) return set_error(IFX_ERR_ARG, "ifx_server_tick: null server");
    const size_t before = V->finished.size();
    ifx_status worst = IFX_OK;
    // issue the steps of every live cohort (up to steps_per_tick, never past the
    // first request to finish); new requests are admitted while those run (the
    // new cohort's set-up overlaps them) and step from the next tick on; then
    // wait for all of them
    const size_t nold = V->cohorts.size();
    for (auto& c : V->cohorts) {
        int k = V->steps_per_tick;
        for (long long id : c.ids) {
            if (id < 0) continue;
            const ifx_server::Request& r = V->reqs[id];
            if (r.state == 1) k = std::min(k, r.nsteps - r.done);
        }
        c.pending = std::max(k, 1);
        ifx_status st = ifx_step_async(c.s, c.pending);
        if (st != IFX_OK) worst = st;
    }
    // cohorts of compatible requests, while requests at the head of the queue
    // fit the budget
    for (int guard = 0; guard < 64 && !V->waiting.empty(); guard++) {
        const size_t nc = V->cohorts.size(), nw = V->waiting.size();
        ifx_status st = admit(V);
        if (st != IFX_OK) worst = st;
        if (V->cohorts.size() == nc && V->waiting.size() == nw) break;
    }
    size_t idx = 0;
    for (auto it = V->cohorts.begin(); it != V->cohorts.end(); idx++) {
        if (idx >= nold) break;  // admitted this tick: no steps yet
        ifx_server::Cohort& c = *it;
        ifx_status st = ifx_step_wait(c.s);
        bool drop = false;
        if (st == IFX_ERR_DIVERGED) {
            // only the requests whose instance diverged fail (the solver retired
            // them); the cohort's other requests go on
            worst = st;
            for (size_t k = 0; k < c.ids.size(); k++) {
                if (c.ids[k] < 0) continue;
                ifx_server::Request& r = V->reqs[c.ids[k]];
                ifx_stats s;
                if (r.state != 1 || ifx_get_stats(c.s, (int)k, &s) != IFX_OK || s.status != IFX_ERR_DIVERGED) continue;
                r.state = 3;
                r.st = s;
                V->finished.push_back(r.id);
                c.live--;
            }
            st = IFX_OK;
        }
        if (st != IFX_OK) {
            worst = st;
            for (long long id : c.ids)
                if (id >= 0 && V->reqs[id].state == 1) {
                    V->reqs[id].state = 3;
                    V->finished.push_back(id);
                }
            drop = true;
        } else {
            for (size_t k = 0; k < c.ids.size(); k++) {
                if (c.ids[k] < 0) continue;
                ifx_server::Request& r = V->reqs[c.ids[k]];
                if (r.state != 1) continue;
                r.done += c.pending;
                if (r.done < r.nsteps) continue;
                const size_t n = (size_t)r.nx * r.ny;
                r.u.resize(n);
                r.v.resize(n);
                r.p.resize(n);
                ifx_status e = ifx_get_field_i(c.s, (int)k, IFX_FIELD_U, r.u.data(), n);
                if (e == IFX_OK) e = ifx_get_field_i(c.s, (int)k, IFX_FIELD_V, r.v.data(), n);
                if (e == IFX_OK) e = ifx_get_field_i(c.s, (int)k, IFX_FIELD_P, r.p.data(), n);
                if (e == IFX_OK) e = ifx_get_stats(c.s, (int)k, &r.st);
                if (e == IFX_OK) e = ifx_set_instance_active(c.s, (int)k, 0);
                r.state = e == IFX_OK ? 2 : 3;
                if (e != IFX_OK) worst = e;
                V->finished.push_back(r.id);
                c.live--;
            }
            drop = c.live == 0;
        }
        if (drop) {
            ifx_destroy(c.s);
            V->used -= std::min(V->used, c.bytes);
            it = V->cohorts.erase(it);
        } else {
            ++it;
        }
    }
    if (n_finished) *n_finished = (int)(V->finished.size() - before);
    return worst;
}

extern "C" ifx_status ifx_server_preempt(ifx_server* V, long long id, int front) {
    if (!V) return set_error(IFX_ERR_ARG, "ifx_server_preempt: null server");
    auto it = V->reqs.find(id);
    if (it == V->reqs.end()) return set_error(IFX_ERR_ARG, "ifx_server_preempt: unknown request");
    ifx_server::Request& r = it->second;
    if (r.state != 1) return set_error(IFX_ERR_STATE, "ifx_server_preempt: request is not running");
    for (auto ci = V->cohorts.begin(); ci != V->cohorts.end(); ++ci) {
        ifx_server::Cohort& c = *ci;
        const auto pos = std::find(c.ids.begin(), c.ids.end(), id);
        if (pos == c.ids.end()) continue;
        const int k = (int)(pos - c.ids.begin());
        size_t nb = 0;
        ifx_status st = ifx_checkpoint_bytes(c.s, k, &nb);
        if (st != IFX_OK) return st;
        r.resume.resize(nb);
        st = ifx_checkpoint_save(c.s, k, r.resume.data(), nb);
        if (st == IFX_OK) st = ifx_set_instance_active(c.s, k, 0);
        if (st != IFX_OK) {
            r.resume.clear();
            return st;
        }
        r.state = 0;
        *pos = -1;  // the slot no longer belongs to the request
        if (front) V->waiting.push_front(id);
        else V->waiting.push_back(id);
        if (--c.live == 0) {
            ifx_destroy(c.s);
            V->used -= std::min(V->used, c.bytes);
            V->cohorts.erase(ci);
        }
        return IFX_OK;
    }
    return set_error(IFX_ERR_STATE, "ifx_server_preempt: request has no cohort");
}

extern "C" ifx_status ifx_server_poll(ifx_server* V, long long* ids, int cap, int* n) {
    if (!V || !n || (cap > 0 && !ids)) return set_error(IFX_ERR_ARG, "ifx_server_poll: bad argument");
    int k = 0;
    while (k < cap && !V->finished.empty()) {
        ids[k++] = V->finished.front();
        V->finished.pop_front();
    }
    *n = k;
    return IFX_OK;
}

extern "C" ifx_status ifx_server_request_state(ifx_server* V, long long id, int* state, int* steps_done, int* nx,
                                               int* ny) {
    if (!V) return set_error(IFX_ERR_ARG, "ifx_server_request_state: null server");
    auto it = V->reqs.find(id);
    if (it == V->reqs.end()) return set_error(IFX_ERR_ARG, "ifx_server_request_state: unknown request");
    if (state) *state = it->second.state;
    if (steps_done) *steps_done = it->second.done;
    if (nx) *nx = it->second.nx;
    if (ny) *ny = it->second.ny;
    return IFX_OK;
}

extern "C" ifx_status ifx_server_result(ifx_server* V, long long id, int field, double* host, size_t n) {
    if (!V || !host) return set_error(IFX_ERR_ARG, "ifx_server_result: bad argument");
    auto it = V->reqs.find(id);
    if (it == V->reqs.end()) return set_error(IFX_ERR_ARG, "ifx_server_result: unknown request");
    const ifx_server::Request& r = it->second;
    if (r.state != 2) return set_error(IFX_ERR_STATE, "ifx_server_result: request has not finished");
    const std::vector<double>* src = field == IFX_FIELD_U ? &r.u : field == IFX_FIELD_V ? &r.v : field == IFX_FIELD_P ? &r.p : nullptr;
    if (!src) return set_error(IFX_ERR_ARG, "ifx_server_result: fields U, V and P are kept");
    if (n < src->size()) return set_error(IFX_ERR_ARG, "ifx_server_result: buffer too small");
    std::memcpy(host, src->data(), src->size() * sizeof(double));
    return IFX_OK;
}

extern "C" ifx_status ifx_server_request_stats(ifx_server* V, long long id, ifx_stats* out) {
    if (!V || !out) return set_error(IFX_ERR_ARG, "ifx_server_request_stats: bad argument");
    auto it = V->reqs.find(id);
    if (it == V->reqs.end()) return set_error(IFX_ERR_ARG, "ifx_server_request_stats: unknown request");
    if (it->second.state != 2) return set_error(IFX_ERR_STATE, "ifx_server_request_stats: request has not finished");
    *out = it->second.st;
    return IFX_OK;
}

extern "C" ifx_status ifx_server_release(ifx_server* V, long long id) {
    if (!V) return set_error(IFX_ERR_ARG, "ifx_server_release: null server");
    auto it = V->reqs.find(id);
    if (it == V->reqs.end()) return set_error(IFX_ERR_ARG, "ifx_server_release: unknown request");
    if (it->second.state < 2) return set_error(IFX_ERR_STATE, "ifx_server_release: request still queued or running");
    V->reqs.erase(it);
    return IFX_OK;
}

extern "C" ifx_status ifx_server_info(ifx_server* V, int* waiting, int* running, int* cohorts, size_t* used_bytes) {
    if (!V) return set_error(IFX_ERR_ARG, "ifx_server_info: null server");
    int run = 0;
    for (const auto& c : V->cohorts) run += c.live;
    if (waiting) *waiting = (int)V->waiting.size();
    if (running) *running = run;
    if (cohorts) *cohorts = (int)V->cohorts.size();
    if (used_bytes) *used_bytes = V->used;
    return IFX_OK;
}

extern "C" void ifx_server_destroy(ifx_server* V) {
    if (!V) return;
    for (auto& c : V->cohorts) ifx_destroy(c.s);
    delete V;
}
