/*
 * Request loop for many independent runs on one GPU (the C ABI of picgb.h,
 * pgb_server_*).  The reference runs one simulation per process
 * (main.cpp, pic.cpp:1040-1279); a request here is that whole run:
 * pic::pic from a restart state, the boundary pass before the loop, and
 * nsteps iterations of pic_run's loop body.
 *
 * Continuous batching.  A round admits queued requests in submission
 * order, first fit, while their pgb_footprint fits the HBM budget and
 * fewer than max_active runs are resident; gives every resident run that
 * is idle its next chunk of at most round_steps steps (pgb_step_async: the
 * run's own stream, so the chunks of all runs overlap on the GPU); waits
 * until at least one chunk has finished; and retires the runs that are
 * done, keeping their particles and counters on the host until they are
 * taken.  No run waits for another: a small run steps at its own pace
 * beside a large one, and a run that finishes frees its memory for the
 * queue at once.  Runs never share device state, so a request's result
 * does not depend on the requests it ran with.
 */
#include <algorithm>
#include <chrono>
#include <cstring>
#include <deque>
#include <map>
#include <string>
#include <thread>
#include <utility>
#include <vector>
#include "picgb.h"

void pgb_set_unbound_error(const std::string& msg);   /* pgb_last_error(NULL) */

namespace {

using Clock = std::chrono::steady_clock;

double seconds_between(Clock::time_point a, Clock::time_point b) {
    return std::chrono::duration<double>(b - a).count();
}

struct Request {
    int64_t id = 0;
    pgb_params p{};
    std::vector<double> e, i;     /* initial particles, 6 doubles each */
    int32_t nsteps = 0;
    int64_t footprint = 0;
    Clock::time_point submitted;
};

struct Resident {
    Request req;
    pgb_run* run = nullptr;
    int32_t done = 0;              /* steps finished                        */
    int32_t inflight = 0;          /* steps of the chunk on the GPU (0: idle) */
    int64_t n_before = -1;         /* particles when the chunk was issued (-1: not read yet) */
    Clock::time_point issued;
};

struct Result {
    std::vector<double> e, i;
    pgb_counters counters{};
};

/* p-quantile of values weighted by counts */
double weighted_quantile(std::vector<std::pair<double, int64_t>> v, double q) {
    if (v.empty()) return 0.0;
    std::sort(v.begin(), v.end());
    int64_t total = 0;
    for (auto& x : v) total += x.second;
    const double target = q * (double)total;
    int64_t acc = 0;
    for (auto& x : v) {
        acc += x.second;
        if ((double)acc >= target) return x.first;
    }
    return v.back().first;
}

int fail(const std::string& msg, int code) {
    pgb_set_unbound_error(msg);
    return code;
}

}  // namespace

struct pgb_server {
    int64_t budget = 0, in_use = 0;
    int32_t round_steps = 1, max_active = 1;
    int64_t next_id = 1;
    std::deque<Request> queue;
    std::vector<Resident> resident;
    std::map<int64_t, Result> results;
    std::deque<int64_t> done_ids;
    int64_t submitted = 0, admitted = 0, completed = 0, run_steps = 0;
    double particle_steps = 0.0, busy = 0.0, t_admit = 0.0, t_retire = 0.0, t_issue = 0.0;
    std::vector<std::pair<double, int64_t>> step_ms;   /* (ms per step, steps) per finished chunk */
    std::vector<std::pair<double, int64_t>> ttc;       /* (seconds, 1) per request */
};

extern "C" int pgb_server_create(int64_t hbm_budget_bytes, int32_t round_steps, int32_t max_active, pgb_server** out) {
    if (!out || hbm_budget_bytes <= 0 || round_steps < 1 || max_active < 1)
        return fail("pgb_server_create: bad argument", PGB_ERR_ARG);
    pgb_server* s = new pgb_server();
    s->budget = hbm_budget_bytes;
    s->round_steps = round_steps;
    s->max_active = max_active;
    *out = s;
    return 0;
}

extern "C" int pgb_server_destroy(pgb_server* s) {
    if (!s) return 0;
    for (auto& r : s->resident) pgb_destroy(r.run);
    delete s;
    return 0;
}

extern "C" int pgb_server_submit(pgb_server* s, const pgb_params* p, const double* e_aos6, int64_t ne,
                                 const double* i_aos6, int64_t ni, int32_t nsteps, int64_t* request_id) {
    if (!s || !p || ne < 0 || ni < 0 || nsteps < 0 || (ne > 0 && !e_aos6) || (ni > 0 && !i_aos6))
        return fail("pgb_server_submit: bad argument", PGB_ERR_ARG);
    Request q;
    q.p = *p;
    q.e.assign(e_aos6, e_aos6 + 6 * ne);
    q.i.assign(i_aos6, i_aos6 + 6 * ni);
    q.nsteps = nsteps;
    int rc = pgb_footprint(p, ne, ni, &q.footprint);
    if (rc) return rc;
    if (q.footprint > s->budget)
        return fail("pgb_server_submit: the run needs " + std::to_string(q.footprint) +
                        " device bytes, more than the server's budget of " + std::to_string(s->budget),
                    PGB_ERR_CAPACITY);
    q.id = s->next_id++;
    q.submitted = Clock::now();
    if (request_id) *request_id = q.id;
    s->queue.push_back(std::move(q));
    s->submitted++;
    return 0;
}

/* create, load and run the pre-loop boundary pass of one admitted request */
static int start_run(Resident& r) {
    int rc = pgb_create(&r.req.p, &r.run);
    if (rc) return rc;
    const int64_t ne = (int64_t)(r.req.e.size() / 6), ni = (int64_t)(r.req.i.size() / 6);
    if ((rc = pgb_load_species(r.run, PGB_ELECTRONS, r.req.e.data(), ne)) ||
        (rc = pgb_load_species(r.run, PGB_IONS, r.req.i.data(), ni)) || (rc = pgb_initial_boundary(r.run))) {
        pgb_set_unbound_error(pgb_last_error(r.run));
        pgb_destroy(r.run);
        r.run = nullptr;
        return rc;
    }
    std::vector<double>().swap(r.req.e);   /* the state now lives on the device */
    std::vector<double>().swap(r.req.i);
    return 0;
}

static int retire(pgb_server* s, Resident& r) {
    Result res;
    int64_t ne = 0, ni = 0;
    int rc;
    if ((rc = pgb_species_count(r.run, PGB_ELECTRONS, &ne)) || (rc = pgb_species_count(r.run, PGB_IONS, &ni)))
        return rc;
    res.e.resize((size_t)(6 * ne));
    res.i.resize((size_t)(6 * ni));
    int64_t got = 0;
    if ((rc = pgb_dump_species(r.run, PGB_ELECTRONS, res.e.data(), ne, &got)) ||
        (rc = pgb_dump_species(r.run, PGB_IONS, res.i.data(), ni, &got)) ||
        (rc = pgb_get_counters(r.run, &res.counters)))
        return rc;
    pgb_destroy(r.run);
    r.run = nullptr;
    s->in_use -= r.req.footprint;
    s->results[r.req.id] = std::move(res);
    s->done_ids.push_back(r.req.id);
    s->completed++;
    s->ttc.push_back({seconds_between(r.req.submitted, Clock::now()), 1});
    return 0;
}

static int64_t particles_of(pgb_run* run) {
    int64_t a = 0, b = 0;
    pgb_species_count(run, PGB_ELECTRONS, &a);
    pgb_species_count(run, PGB_IONS, &b);
    return a + b;
}

extern "C" int pgb_server_round(pgb_server* s, int32_t* completed) {
    if (!s) return fail("pgb_server_round: bad argument", PGB_ERR_ARG);
    if (completed) *completed = 0;
    const Clock::time_point t0 = Clock::now();
    /* admission: first fit in submission order */
    for (auto it = s->queue.begin(); it != s->queue.end() && (int32_t)s->resident.size() < s->max_active;) {
        if (s->in_use + it->footprint > s->budget) {
            ++it;
            continue;
        }
        Resident r;
        r.req = std::move(*it);
        it = s->queue.erase(it);
        const Clock::time_point ta = Clock::now();
        int rc = start_run(r);
        s->t_admit += seconds_between(ta, Clock::now());
        if (rc) return fail("pgb_server_round: starting request " + std::to_string(r.req.id) + " failed: " +
                                pgb_last_error(nullptr), rc);
        s->in_use += r.req.footprint;
        s->admitted++;
        s->resident.push_back(std::move(r));
    }
    /* every idle run gets its next chunk */
    int inflight = 0;
    const Clock::time_point ti = Clock::now();
    for (auto& r : s->resident) {
        if (r.inflight == 0 && r.done < r.req.nsteps) {
            const int32_t k = std::min(s->round_steps, r.req.nsteps - r.done);
            if (r.n_before < 0) r.n_before = particles_of(r.run);
            r.issued = Clock::now();
            int rc = pgb_step_async(r.run, k);
            if (rc) return fail("pgb_server_round: stepping request " + std::to_string(r.req.id) + " failed: " +
                                    pgb_last_error(r.run), rc);
            r.inflight = k;
        }
        if (r.inflight) inflight++;
    }
    s->t_issue += seconds_between(ti, Clock::now());
    /* wait until at least one chunk has finished */
    bool any = false;
    while (inflight > 0 && !any) {
        for (auto& r : s->resident) {
            if (!r.inflight) continue;
            int32_t idle = 0;
            int rc = pgb_query(r.run, &idle);
            if (rc) return fail("pgb_server_round: request " + std::to_string(r.req.id) + " failed: " +
                                    pgb_last_error(r.run), rc);
            if (!idle) continue;
            const double ms = 1000.0 * seconds_between(r.issued, Clock::now()) / r.inflight;
            s->step_ms.push_back({ms, (int64_t)r.inflight});
            const int64_t n_after = particles_of(r.run);
            s->particle_steps += 0.5 * (double)(r.n_before + n_after) * r.inflight;
            r.n_before = n_after;   /* the next chunk starts from here */
            s->run_steps += r.inflight;
            r.done += r.inflight;
            r.inflight = 0;
            any = true;
        }
        if (!any) std::this_thread::sleep_for(std::chrono::microseconds(20));
    }
    /* retire the finished runs */
    for (size_t j = 0; j < s->resident.size();) {
        Resident& r = s->resident[j];
        if (r.inflight == 0 && r.done >= r.req.nsteps) {
            const Clock::time_point tr = Clock::now();
            int rc = retire(s, r);
            s->t_retire += seconds_between(tr, Clock::now());
            if (rc) return rc;
            if (completed) (*completed)++;
            s->resident.erase(s->resident.begin() + (long)j);
        } else {
            ++j;
        }
    }
    s->busy += seconds_between(t0, Clock::now());
    return 0;
}

extern "C" int pgb_server_done(pgb_server* s, int64_t* ids, int32_t cap, int32_t* n_out) {
    if (!s || !n_out || cap < 0 || (cap > 0 && !ids)) return fail("pgb_server_done: bad argument", PGB_ERR_ARG);
    int32_t n = 0;
    while (n < cap && !s->done_ids.empty()) {
        ids[n++] = s->done_ids.front();
        s->done_ids.pop_front();
    }
    *n_out = n;
    return 0;
}

extern "C" int pgb_server_result_size(pgb_server* s, int64_t id, int64_t* ne, int64_t* ni) {
    if (!s || !ne || !ni) return fail("pgb_server_result_size: bad argument", PGB_ERR_ARG);
    auto it = s->results.find(id);
    if (it == s->results.end()) return fail("pgb_server_result_size: no finished request with this id", PGB_ERR_STATE);
    *ne = (int64_t)(it->second.e.size() / 6);
    *ni = (int64_t)(it->second.i.size() / 6);
    return 0;
}

extern "C" int pgb_server_result(pgb_server* s, int64_t id, double* e_aos6, int64_t cap_e, double* i_aos6,
                                 int64_t cap_i, pgb_counters* counters) {
    if (!s || cap_e < 0 || cap_i < 0 || (cap_e > 0 && !e_aos6) || (cap_i > 0 && !i_aos6))
        return fail("pgb_server_result: bad argument", PGB_ERR_ARG);
    auto it = s->results.find(id);
    if (it == s->results.end()) return fail("pgb_server_result: no finished request with this id", PGB_ERR_STATE);
    const Result& r = it->second;
    const size_t ce = std::min<size_t>(r.e.size(), (size_t)(6 * cap_e)), ci = std::min<size_t>(r.i.size(), (size_t)(6 * cap_i));
    if (ce) std::memcpy(e_aos6, r.e.data(), sizeof(double) * ce);
    if (ci) std::memcpy(i_aos6, r.i.data(), sizeof(double) * ci);
    if (counters) *counters = r.counters;
    s->results.erase(it);
    return 0;
}

extern "C" int pgb_server_get_stats(pgb_server* s, pgb_server_stats* out) {
    if (!s || !out) return fail("pgb_server_get_stats: bad argument", PGB_ERR_ARG);
    std::memset(out, 0, sizeof(*out));
    out->submitted = s->submitted;
    out->admitted = s->admitted;
    out->completed = s->completed;
    out->active = (int64_t)s->resident.size();
    out->queued = (int64_t)s->queue.size();
    out->run_steps = s->run_steps;
    out->particle_steps = s->particle_steps;
    out->busy_seconds = s->busy;
    out->step_ms_p50 = weighted_quantile(s->step_ms, 0.50);
    out->step_ms_p99 = weighted_quantile(s->step_ms, 0.99);
    out->ttc_s_p50 = weighted_quantile(s->ttc, 0.50);
    out->ttc_s_p99 = weighted_quantile(s->ttc, 0.99);
    out->hbm_in_use = s->in_use;
    out->hbm_budget = s->budget;
    out->admit_seconds = s->t_admit;
    out->retire_seconds = s->t_retire;
    out->issue_seconds = s->t_issue;
    return 0;
}
