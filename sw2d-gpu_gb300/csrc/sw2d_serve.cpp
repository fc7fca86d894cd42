// sw2d_serve.cpp -- continuous batching over one batch (the sw2d_server_*
// calls of include/sw2d.h): host C++ on top of the batch's C ABI.
//
// Requests wait in submission order.  A round (sw2d_server_step) admits
// every waiting request that finds a free scenario slot and fits the
// batch's memory budget -- one that does not fit keeps its place, and
// smaller ones behind it may pass it, so memory freed by a retirement is
// used at once --, advances the resident requests by one tick of
// launches_per_step iterations, then polls the batch (which waits for the
// tick) and retires the requests whose plan has stopped: budgets and depth
// are copied to host memory and the scenario leaves the batch, returning its
// memory in stream order.  The numerics are the batch's: each request
// advances exactly as it would alone.
#include <cstring>
#include <deque>
#include <map>
#include <new>
#include <string>
#include <vector>

#include "sw2d.h"

namespace {

struct ServeRequest {
    int32_t state = SW2D_REQ_PENDING;
    sw2d_config cfg;
    std::vector<double> z, manning, depth, rain;  // inputs, kept until admission
    int32_t rain_kind = SW2D_RAIN_NONE, n_rain = 0;
    double rain_dt = 1.0, t_end = 0.0;
    int64_t bytes = 0;     // device footprint in the batch
    int32_t scenario = -1; // batch scenario id while resident
    double t = 0.0;        // simulated time and iterations, as of the last poll
    int64_t steps = 0;
    sw2d_budget budget;    // final budgets (done)
    std::vector<double> result;  // final depth raster (done, keep_depth)
    std::string error;     // why the batch refused it (failed)

    void drop_inputs() {
        std::vector<double>().swap(z);
        std::vector<double>().swap(manning);
        std::vector<double>().swap(depth);
        std::vector<double>().swap(rain);
    }
};

}  // namespace

struct sw2d_server {
    sw2d_server_config cfg;
    sw2d_batch *batch = nullptr;
    std::map<int32_t, ServeRequest> req;  // by request id
    std::deque<int32_t> pending;          // request ids in submission order
    std::map<int32_t, int32_t> resident;  // batch scenario id -> request id
    int64_t bytes_used = 0;
    int32_t next_id = 1;
    std::string err;
    // sw2d_batch_poll's outputs
    std::vector<int32_t> p_ids, p_run;
    std::vector<double> p_t;
    std::vector<int64_t> p_steps;
};

namespace {

int sfail(sw2d_server *s, int code, const std::string &msg) {
    if (s) s->err = msg;
    return code;
}

// The batch's status with its message, as the server's.
int from_batch(sw2d_server *s, int code, const char *what) {
    return sfail(s, code, std::string(what) + ": " + sw2d_batch_last_error(s->batch));
}

const ServeRequest *find(const sw2d_server *s, int32_t id) {
    auto it = s->req.find(id);
    return it == s->req.end() ? nullptr : &it->second;
}

// Admission in submission order while slots and memory allow.
int admit(sw2d_server *s) {
    const int64_t budget = s->cfg.batch.max_bytes;
    for (auto it = s->pending.begin(); it != s->pending.end();) {
        ServeRequest &r = s->req[*it];
        const bool slot = (int64_t)s->resident.size() < (int64_t)s->cfg.batch.max_scenarios;
        if (!slot) break;  // no request can enter before a retirement
        if (budget > 0 && s->bytes_used + r.bytes > budget) {
            ++it;  // waits for memory and keeps its place
            continue;
        }
        int32_t sid = -1;
        const int rc = sw2d_batch_add(s->batch, &r.cfg, r.z.data(), r.manning.empty() ? nullptr : r.manning.data(),
                                      r.depth.data(), r.rain_kind, r.rain.empty() ? nullptr : r.rain.data(),
                                      r.n_rain, r.rain_dt, r.t_end, &sid);
        if (rc == SW2D_ERR_INVALID_ARG || rc == SW2D_ERR_OOM) {  // refused: this request fails alone
            r.state = SW2D_REQ_FAILED;
            r.error = sw2d_batch_last_error(s->batch);
        } else if (rc != SW2D_OK) {
            return from_batch(s, rc, "admission");  // the device failed: the request keeps its place
        } else {
            r.state = SW2D_REQ_RUNNING;
            r.scenario = sid;
            s->resident[sid] = *it;
            s->bytes_used += r.bytes;
        }
        r.drop_inputs();  // the batch holds its own copy (sw2d_batch_add waits for its uploads)
        it = s->pending.erase(it);
    }
    return SW2D_OK;
}

// Polls the batch (waiting for the queued tick) and retires the requests
// whose plan has stopped.
int retire(sw2d_server *s) {
    const size_t cap = s->resident.size();
    if (cap == 0) return SW2D_OK;
    s->p_ids.resize(cap);
    s->p_run.resize(cap);
    s->p_t.resize(cap);
    s->p_steps.resize(cap);
    int32_t n = 0;
    int rc = sw2d_batch_poll(s->batch, s->p_ids.data(), s->p_run.data(), s->p_t.data(), s->p_steps.data(),
                             (int32_t)cap, &n);
    if (rc) return from_batch(s, rc, "poll");
    for (int32_t k = 0; k < n; k++) {
        auto it = s->resident.find(s->p_ids[k]);
        if (it == s->resident.end()) continue;
        ServeRequest &r = s->req[it->second];
        r.t = s->p_t[k];
        r.steps = s->p_steps[k];
        if (s->p_run[k]) continue;
        rc = sw2d_batch_get_budget(s->batch, r.scenario, &r.budget);
        if (rc) return from_batch(s, rc, "budget");
        if (s->cfg.keep_depth) {
            try {
                r.result.resize((size_t)r.cfg.rows * r.cfg.cols);
            } catch (...) {  // the request stays resident; a later step retries
                return sfail(s, SW2D_ERR_OOM, "host memory for a finished request's depth");
            }
            rc = sw2d_batch_get_field(s->batch, r.scenario, SW2D_FIELD_DEPTH, r.result.data());
            if (rc) return from_batch(s, rc, "depth");
        }
        rc = sw2d_batch_remove(s->batch, r.scenario);
        if (rc) return from_batch(s, rc, "retire");
        s->bytes_used -= r.bytes;
        r.state = SW2D_REQ_DONE;
        r.scenario = -1;
        s->resident.erase(it);
    }
    return SW2D_OK;
}

}  // namespace

extern "C" {

int sw2d_server_config_init(sw2d_server_config *cfg) {
    if (!cfg) return SW2D_ERR_INVALID_ARG;
    std::memset(cfg, 0, sizeof(*cfg));
    sw2d_batch_config_init(&cfg->batch);
    cfg->launches_per_step = 24;
    cfg->keep_depth = 1;
    return SW2D_OK;
}

int sw2d_server_create(const sw2d_server_config *cfg, sw2d_server **out) {
    if (!cfg || !out) return SW2D_ERR_INVALID_ARG;
    *out = nullptr;
    if (cfg->launches_per_step < 1 || (cfg->keep_depth != 0 && cfg->keep_depth != 1)) return SW2D_ERR_INVALID_ARG;
    sw2d_server *s = new (std::nothrow) sw2d_server();
    if (!s) return SW2D_ERR_OOM;
    s->cfg = *cfg;
    const int rc = sw2d_batch_create(&cfg->batch, &s->batch);
    if (rc) {
        delete s;
        return rc;
    }
    *out = s;
    return SW2D_OK;
}

int sw2d_server_destroy(sw2d_server *s) {
    if (!s) return SW2D_ERR_INVALID_ARG;
    const int rc = s->batch ? sw2d_batch_destroy(s->batch) : SW2D_OK;
    delete s;
    return rc;
}

int sw2d_server_submit(sw2d_server *s, const sw2d_config *cfg, const double *z, const double *manning,
                       const double *depth, int32_t rain_kind, const double *rain, int32_t n_rain, double rain_dt,
                       double t_end, int32_t *request) {
    if (!s || !cfg || !z || !depth || !request) return sfail(s, SW2D_ERR_INVALID_ARG, "null argument");
    if (cfg->precision != SW2D_PREC_F32 || cfg->dt_mode != SW2D_DT_CFL)
        return sfail(s, SW2D_ERR_INVALID_ARG, "served requests are FP32 with the CFL rule");
    if (rain_kind != SW2D_RAIN_NONE && (!rain || n_rain < 1))
        return sfail(s, SW2D_ERR_INVALID_ARG, "bad rain series");
    const int32_t nr = rain_kind == SW2D_RAIN_NONE ? 0 : n_rain;
    int64_t bytes = 0;
    if (sw2d_batch_scenario_bytes(cfg, nr, manning != nullptr, &bytes) != SW2D_OK)
        return sfail(s, SW2D_ERR_INVALID_ARG, "bad grid size");
    if (s->cfg.batch.max_bytes > 0 && bytes > s->cfg.batch.max_bytes)
        return sfail(s, SW2D_ERR_INVALID_ARG, "the request needs more device memory than the whole budget");
    const size_t cells = (size_t)cfg->rows * cfg->cols;
    const int32_t id = s->next_id;
    try {  // no exception crosses the C ABI: a failed host copy is SW2D_ERR_OOM
        ServeRequest r;
        r.cfg = *cfg;
        r.z.assign(z, z + cells);
        if (manning) r.manning.assign(manning, manning + cells);
        r.depth.assign(depth, depth + cells);
        if (nr > 0) r.rain.assign(rain, rain + nr);
        r.rain_kind = rain_kind;
        r.n_rain = nr;
        r.rain_dt = rain_dt;
        r.t_end = t_end;
        r.bytes = bytes;
        std::memset(&r.budget, 0, sizeof(r.budget));
        s->req[id] = std::move(r);
        s->pending.push_back(id);
    } catch (...) {
        s->req.erase(id);
        return sfail(s, SW2D_ERR_OOM, "host memory for the request's copy");
    }
    s->next_id++;
    *request = id;
    return SW2D_OK;
}

int sw2d_server_step(sw2d_server *s, int32_t *pending, int32_t *running) {
    if (!s) return SW2D_ERR_INVALID_ARG;
    try {  // no exception crosses the C ABI (host allocations of the bookkeeping)
        int rc = admit(s);
        if (rc) return rc;
        if (!s->resident.empty()) {
            rc = sw2d_batch_advance(s->batch, s->cfg.launches_per_step, nullptr);
            if (rc) return from_batch(s, rc, "advance");
            rc = retire(s);
            if (rc) return rc;
        }
    } catch (...) {
        return SW2D_ERR_OOM;
    }
    if (pending) *pending = (int32_t)s->pending.size();
    if (running) *running = (int32_t)s->resident.size();
    return SW2D_OK;
}

int sw2d_server_poll(const sw2d_server *s, int32_t request, int32_t *state, double *t, int64_t *steps) {
    if (!s || !state) return SW2D_ERR_INVALID_ARG;
    const ServeRequest *r = find(s, request);
    *state = r ? r->state : SW2D_REQ_UNKNOWN;
    if (t) *t = r ? r->t : 0.0;
    if (steps) *steps = r ? r->steps : 0;
    return SW2D_OK;
}

int sw2d_server_get_budget(const sw2d_server *s, int32_t request, sw2d_budget *out) {
    if (!s || !out) return SW2D_ERR_INVALID_ARG;
    const ServeRequest *r = find(s, request);
    if (!r || r->state != SW2D_REQ_DONE) return SW2D_ERR_INVALID_ARG;
    *out = r->budget;
    return SW2D_OK;
}

int sw2d_server_get_depth(const sw2d_server *s, int32_t request, double *out) {
    if (!s || !out) return SW2D_ERR_INVALID_ARG;
    const ServeRequest *r = find(s, request);
    if (!r || r->state != SW2D_REQ_DONE || r->result.empty()) return SW2D_ERR_INVALID_ARG;
    std::memcpy(out, r->result.data(), r->result.size() * sizeof(double));
    return SW2D_OK;
}

int sw2d_server_cancel(sw2d_server *s, int32_t request) {
    if (!s) return SW2D_ERR_INVALID_ARG;
    auto it = s->req.find(request);
    if (it == s->req.end()) return sfail(s, SW2D_ERR_INVALID_ARG, "unknown request");
    ServeRequest &r = it->second;
    if (r.state == SW2D_REQ_PENDING) {
        for (auto p = s->pending.begin(); p != s->pending.end(); ++p)
            if (*p == request) {
                s->pending.erase(p);
                break;
            }
        r.drop_inputs();
    } else if (r.state == SW2D_REQ_RUNNING) {
        const int rc = sw2d_batch_remove(s->batch, r.scenario);
        if (rc) return from_batch(s, rc, "cancel");
        s->resident.erase(r.scenario);
        s->bytes_used -= r.bytes;
        r.scenario = -1;
    } else {
        return sfail(s, SW2D_ERR_INVALID_ARG, "the request is not pending or running");
    }
    r.state = SW2D_REQ_CANCELLED;
    return SW2D_OK;
}

int sw2d_server_release(sw2d_server *s, int32_t request) {
    if (!s) return SW2D_ERR_INVALID_ARG;
    auto it = s->req.find(request);
    if (it == s->req.end()) return sfail(s, SW2D_ERR_INVALID_ARG, "unknown request");
    const int32_t st = it->second.state;
    if (st != SW2D_REQ_DONE && st != SW2D_REQ_FAILED && st != SW2D_REQ_CANCELLED)
        return sfail(s, SW2D_ERR_INVALID_ARG, "the request has not finished");
    s->req.erase(it);
    return SW2D_OK;
}

int sw2d_server_bytes_in_use(const sw2d_server *s, int64_t *bytes) {
    if (!s || !bytes) return SW2D_ERR_INVALID_ARG;
    *bytes = s->bytes_used;
    return SW2D_OK;
}

int sw2d_server_get_batch(sw2d_server *s, sw2d_batch **batch) {
    if (!s || !batch) return SW2D_ERR_INVALID_ARG;
    *batch = s->batch;
    return SW2D_OK;
}

const char *sw2d_server_last_error(const sw2d_server *s) { return s ? s->err.c_str() : "null server"; }

const char *sw2d_server_request_error(const sw2d_server *s, int32_t request) {
    if (!s) return "";
    const ServeRequest *r = find(s, request);
    return r ? r->error.c_str() : "";
}

}  // extern "C"
