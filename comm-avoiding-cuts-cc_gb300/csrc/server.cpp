// Serving loop: square_root, approx_cut and parallel_cc queries answered as they arrive from
// graphs resident in HBM, with continuous batching of the Karger-Stein work.
//
// The reference answers one query per process launch (src/executables/*.cpp). A cac_server owns
// three contexts on one device, each with its own CUDA stream:
//   - the upload context, used under a lock by cac_server_graph on the caller's thread;
//   - the cut worker: a thread driving one persistent Karger-Stein engine. Before every engine
//     step it admits waiting square_root queries (Stage 1 and the dense roots) while the
//     estimated footprint of the running ones fits the budget; the step then contracts,
//     quotients and solves the leaves of every running query together, so a query that arrives
//     while others are on the GPU joins their launches instead of waiting behind them. A query
//     is finished when none of its nodes is left; its trial cuts are reduced on the host;
//   - the graph worker: a thread running parallel_cc and approx_cut queries on its own stream,
//     concurrently with the cut worker's launches.
// A response does not depend on what else is in flight: every random draw of a query is
// addressed by its own (seed + rank, trial, node, round, draw) key and every trial writes its
// own cut slot.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstdio>
#include <deque>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "cac_internal.h"

using namespace cac;

namespace {

using Clock = std::chrono::steady_clock;

double ms_between(Clock::time_point a, Clock::time_point b) {
    return std::chrono::duration<double, std::milli>(b - a).count();
}

struct Request {
    uint64_t ticket = 0;
    cac_request req{};
    cac_response resp{};
    bool done = false;
    Clock::time_point t_submit, t_admit;
    // square_root state
    uint32_t ranks = 1, per_rank = 0, groups = 0, query = 0;
    uint64_t trials = 0, est_bytes = 0;
    void *d_cuts = nullptr;
    int st = CAC_OK;  // an admission error, reported when the query's nodes have drained
    std::string msg;
};

}  // namespace

struct cac_server {
    cac_ctx *up = nullptr;
    cac_ctx *cut = nullptr;
    cac_ctx *graph = nullptr;
    uint64_t budget = 0;
    std::mutex mu;  // guards the queues, the request table and `stop`
    std::condition_variable cv_work, cv_done;
    std::deque<Request *> cut_queue, graph_queue;
    std::unordered_map<uint64_t, std::unique_ptr<Request>> requests;
    uint64_t next_ticket = 1;
    bool stop = false;
    std::mutex up_mu;
    std::thread cut_thread, graph_thread;
};

namespace {

void finish(cac_server *s, Request *r, int status, const std::string &msg) {
    const Clock::time_point now = Clock::now();
    std::lock_guard<std::mutex> lk(s->mu);
    r->resp.status = status;
    r->resp.queue_ms = ms_between(r->t_submit, r->t_admit);
    r->resp.service_ms = ms_between(r->t_admit, now);
    if (status != CAC_OK) std::snprintf(r->resp.message, sizeof(r->resp.message), "%s", msg.c_str());
    r->done = true;
    s->cv_done.notify_all();
}

int run_cc(cac_ctx *ctx, Request *r) {
    const cac_graph *g = r->req.graph;
    cac_cc_result cr{};
    void *d_labels = nullptr;
    if (r->req.labels_host && g->n) CAC_TRY(stream_alloc(ctx, &d_labels, (size_t)g->n * 4));
    int st = cc_run(ctx, g->n, g->m, g->u, g->v, r->req.seed, r->ranks, static_cast<uint32_t *>(d_labels), &cr);
    if (st == CAC_OK && d_labels) {
        if (cudaMemcpyAsync(r->req.labels_host, d_labels, (size_t)g->n * 4, cudaMemcpyDeviceToHost, ctx->stream) !=
                cudaSuccess ||
            cudaStreamSynchronize(ctx->stream) != cudaSuccess) {
            set_error("server: reading parallel_cc labels failed");
            st = CAC_ERR_CUDA;
        }
    }
    if (d_labels) stream_free(ctx, d_labels, (size_t)g->n * 4);
    r->resp.num_components = cr.num_components;
    return st;
}

void graph_worker(cac_server *s) {
    cudaSetDevice(s->graph->device);
    for (;;) {
        Request *r = nullptr;
        {
            std::unique_lock<std::mutex> lk(s->mu);
            s->cv_work.wait(lk, [&] { return s->stop || !s->graph_queue.empty(); });
            if (s->graph_queue.empty()) return;
            r = s->graph_queue.front();
            s->graph_queue.pop_front();
            r->t_admit = Clock::now();
        }
        int st;
        if (r->req.kind == CAC_QUERY_CC) {
            st = run_cc(s->graph, r);
        } else {
            cac_approx_result ar{};
            st = approx_run(s->graph, r->req.graph, r->req.success_probability, r->req.seed, r->ranks, false, &ar);
            r->resp.cut = ar.cut;
            r->resp.trials = ar.trials;
        }
        finish(s, r, st, st == CAC_OK ? std::string() : std::string(cac_last_error()));
    }
}

// The cut worker's state between engine steps.
struct CutWorker {
    cac_server *s;
    std::unique_ptr<KsEngine> eng;
    std::vector<Request *> running;
    std::vector<uint32_t> free_ids;  // engine query ids are recycled
    uint32_t next_id = 0;
    uint64_t held_est = 0;
    bool planning = true;  // levels planned ahead, except while running queries are being redone

    uint32_t take_id() {
        if (!free_ids.empty()) {
            const uint32_t q = free_ids.back();
            free_ids.pop_back();
            return q;
        }
        return next_id++;
    }

    int new_engine() {
        eng.reset(new KsEngine(s->cut));
        eng->set_plan_ahead(planning && s->cut->plan_ahead);
        return eng->init_err();
    }

    // A planned level met a child off its target size. Which running queries it touched is not
    // known, so all of them run again: the engine drains them (their cuts are discarded), its error
    // word is cleared, and they are admitted again with the levels stepped one by one. Planning
    // resumes once the engine is idle. Queries collected earlier were read with a clean error word
    // after a synchronisation, so every kernel of theirs had run without a miss.
    int redo_running() {
        while (!eng->idle()) CAC_TRY(eng->step());
        std::vector<Request *> again;
        for (Request *r : running) {
            free_ids.push_back(r->query);
            if (r->d_cuts) stream_free(s->cut, r->d_cuts, std::max<uint64_t>(r->trials, 1) * 8);
            r->d_cuts = nullptr;
            r->st = CAC_OK;
            r->msg.clear();
            again.push_back(r);
        }
        running.clear();
        CAC_TRY(eng->init_err());
        planning = false;
        eng->set_plan_ahead(false);
        s->cut->plan_redos++;
        admit(again);
        return CAC_OK;
    }

    void retire(Request *r, int st, const std::string &msg) {
        if (r->d_cuts) stream_free(s->cut, r->d_cuts, std::max<uint64_t>(r->trials, 1) * 8);
        r->d_cuts = nullptr;
        held_est -= r->est_bytes;
        free_ids.push_back(r->query);
        finish(s, r, st, msg);
    }

    // Admits the queries taken from the queue together: their Stage 1 trials share launches.
    void admit(const std::vector<Request *> &batch) {
        std::vector<MincutQuery> qs;
        std::vector<uint32_t> ids;
        std::vector<Request *> rs;
        for (Request *r : batch) {
            r->query = take_id();
            running.push_back(r);
            const int st = stream_alloc(s->cut, &r->d_cuts, std::max<uint64_t>(r->trials, 1) * 8);
            if (st != CAC_OK) {
                r->st = st;
                r->msg = cac_last_error();
                continue;
            }
            qs.push_back(MincutQuery{r->req.graph, r->req.seed, r->ranks, r->per_rank,
                                     static_cast<uint64_t *>(r->d_cuts), 0, r->groups});
            ids.push_back(r->query);
            rs.push_back(r);
        }
        if (rs.empty()) return;
        std::vector<int> status;
        std::vector<std::string> msgs;
        mincut_admit_queries(s->cut, *eng, qs, ids, status, msgs);
        for (size_t i = 0; i < rs.size(); i++)
            if (status[i] != CAC_OK) {  // nodes already added still write into d_cuts: report once they drain
                rs[i]->st = status[i];
                rs[i]->msg = msgs[i];
            }
    }

    // Queries with no node left in the engine are finished: reduce their cuts on the host (after a
    // check that no planned level missed its target; if one did, the running queries are redone).
    int collect() {
        bool any_done = false;
        for (const Request *r : running)
            any_done = any_done || !(r->query < eng->outstanding.size() && eng->outstanding[r->query] > 0);
        if (!any_done) return CAC_OK;
        if (planning) {
            uint32_t err = 0;
            CAC_TRY(eng->read_err(&err));
            if (err & kErrPlan) return redo_running();
        }
        for (size_t i = 0; i < running.size();) {
            Request *r = running[i];
            if (r->query < eng->outstanding.size() && eng->outstanding[r->query] > 0) {
                i++;
                continue;
            }
            int st = r->st;
            std::string msg = r->msg;
            if (st == CAC_OK) {
                std::vector<uint64_t> cuts(r->trials);
                uint32_t err = 0;
                if (r->trials && (cudaMemcpyAsync(cuts.data(), r->d_cuts, r->trials * 8, cudaMemcpyDeviceToHost,
                                                  s->cut->stream) != cudaSuccess ||
                                  cudaStreamSynchronize(s->cut->stream) != cudaSuccess)) {
                    st = CAC_ERR_CUDA;
                    msg = "server: reading a query's trial cuts failed";
                } else if (eng->read_err(&err) != CAC_OK || err) {
                    st = engine_error(err);
                    msg = cac_last_error();
                } else {
                    uint64_t md = 0;
                    if (graph_min_degree(s->cut, const_cast<cac_graph *>(r->req.graph), &md) != CAC_OK) {
                        st = CAC_ERR_CUDA;
                        msg = "server: the graph's minimum weighted degree could not be computed";
                    } else {
                        r->resp.cut = r->trials ? std::min(md, *std::min_element(cuts.begin(), cuts.end())) : 0;
                        r->resp.trials = r->per_rank;
                    }
                }
            }
            running[i] = running.back();
            running.pop_back();
            retire(r, st, msg);
        }
        return CAC_OK;
    }

    void fail_all(int st, const std::string &msg) {
        eng.reset();  // synchronises the stream and frees the engine's buffers
        for (Request *r : running) retire(r, st, msg);
        running.clear();
        free_ids.clear();
        next_id = 0;
    }

    // Without an engine nothing can run: every waiting query fails, now and until shutdown.
    void fail_queue(const std::string &msg) {
        for (;;) {
            Request *r = nullptr;
            {
                std::unique_lock<std::mutex> lk(s->mu);
                s->cv_work.wait(lk, [&] { return s->stop || !s->cut_queue.empty(); });
                if (s->cut_queue.empty()) return;
                r = s->cut_queue.front();
                s->cut_queue.pop_front();
                r->t_admit = Clock::now();
            }
            finish(s, r, CAC_ERR_CUDA, msg);
        }
    }

    void loop() {
        cudaSetDevice(s->cut->device);
        if (new_engine() != CAC_OK) {
            fail_queue(cac_last_error());
            return;
        }
        for (;;) {
            std::vector<Request *> batch;
            {
                std::unique_lock<std::mutex> lk(s->mu);
                s->cv_work.wait(lk, [&] { return s->stop || !s->cut_queue.empty() || !running.empty(); });
                if (s->cut_queue.empty() && running.empty()) return;  // stop requested, nothing left
                while (!s->cut_queue.empty()) {
                    Request *r = s->cut_queue.front();
                    const bool alone = running.empty() && batch.empty();
                    if (!alone && s->budget && held_est + r->est_bytes > s->budget) break;
                    s->cut_queue.pop_front();
                    held_est += r->est_bytes;
                    r->t_admit = Clock::now();
                    batch.push_back(r);
                }
            }
            if (!batch.empty()) admit(batch);
            int st = eng->idle() ? CAC_OK : eng->step();
            if (st == CAC_OK) st = collect();
            if (st != CAC_OK) {
                fail_all(st, cac_last_error());
                if (new_engine() != CAC_OK) {
                    fail_queue(cac_last_error());
                    return;
                }
                continue;
            }
            if (!planning && running.empty() && eng->idle()) {  // the redone queries are through
                planning = true;
                eng->set_plan_ahead(s->cut->plan_ahead);
            }
        }
    }
};

void cut_worker(cac_server *s) {
    CutWorker w{s, nullptr, {}, {}, 0, 0};
    w.loop();
    w.eng.reset();
}

}  // namespace

extern "C" {

int cac_server_create(const cac_server_config *config, cac_server **out) {
    if (!out) {
        set_error("cac_server_create: out is NULL");
        return CAC_ERR_INVALID;
    }
    *out = nullptr;
    cac_server_config cfg{};
    if (config) cfg = *config;
    auto *s = new cac_server();
    s->budget = cfg.hbm_budget_bytes;
    cac_config c{cfg.device, nullptr, 0};
    cac_config cc{cfg.device, nullptr, cfg.hbm_budget_bytes};  // the engine's buffers count against the budget
    int st = cac_ctx_create(&c, &s->up);
    if (st == CAC_OK) st = cac_ctx_create(&cc, &s->cut);
    if (st == CAC_OK) st = cac_ctx_create(&c, &s->graph);
    if (st != CAC_OK) {
        cac_ctx_destroy(s->graph);
        cac_ctx_destroy(s->cut);
        cac_ctx_destroy(s->up);
        delete s;
        return st;
    }
    s->cut_thread = std::thread(cut_worker, s);
    s->graph_thread = std::thread(graph_worker, s);
    *out = s;
    return CAC_OK;
}

int cac_server_graph(cac_server *s, uint32_t n, uint64_t m, const uint32_t *u, const uint32_t *v, const uint32_t *w,
                     cac_graph **out) {
    if (!s) {
        set_error("cac_server_graph: server is NULL");
        return CAC_ERR_INVALID;
    }
    std::lock_guard<std::mutex> lk(s->up_mu);
    cudaSetDevice(s->up->device);
    CAC_TRY(cac_graph_from_edges(s->up, n, m, u, v, w, CAC_HOST, out));
    CAC_CUDA_TRY(cudaStreamSynchronize(s->up->stream));  // visible to the workers' streams
    return CAC_OK;
}

int cac_server_generate(cac_server *s, const cac_gen_spec *spec, cac_graph **out) {
    if (!s) {
        set_error("cac_server_generate: server is NULL");
        return CAC_ERR_INVALID;
    }
    std::lock_guard<std::mutex> lk(s->up_mu);
    cudaSetDevice(s->up->device);
    CAC_TRY(cac_graph_generate(s->up, spec, out));
    CAC_CUDA_TRY(cudaStreamSynchronize(s->up->stream));
    return CAC_OK;
}

int cac_server_submit(cac_server *s, const cac_request *req, uint64_t *ticket) {
    if (!s || !req || !ticket || !req->graph ||
        (req->kind != CAC_QUERY_MINCUT && req->kind != CAC_QUERY_APPROX && req->kind != CAC_QUERY_CC)) {
        set_error("cac_server_submit: invalid request");
        return CAC_ERR_INVALID;
    }
    const cac_graph *g = req->graph;
    auto r = std::make_unique<Request>();
    r->req = *req;
    r->t_submit = Clock::now();
    r->ranks = req->virtual_ranks ? req->virtual_ranks : 1;
    if (req->kind == CAC_QUERY_MINCUT) {
        if (g->n < 2 || !(req->success_probability >= 0.0 && req->success_probability < 1.0)) {
            set_error("cac_server_submit: square_root needs n >= 2 and a success probability in [0, 1)");
            return CAC_ERR_INVALID;
        }
        const uint32_t t = intermediate_size(g->n, g->m);
        if (g->total_weight >= (1ull << 55)) {
            set_error("cac_server_submit: graph outside the supported square_root sizes");
            return CAC_ERR_UNSUPPORTED;
        }
        TrialLayout L{};
        CAC_TRY(trial_layout("cac_server_submit", g->n, g->m, req->success_probability, r->ranks, &L));
        r->per_rank = L.per_rank;
        r->groups = L.high ? L.groups : 0;
        r->trials = L.total;
        const uint64_t tt = std::min<uint64_t>(t, g->n);
        r->est_bytes = (t < g->n ? r->trials : 1) * tt * tt * 8 * 3 + r->trials * 8;
    } else if (req->kind == CAC_QUERY_APPROX &&
               !(req->success_probability > 0.0 && req->success_probability < 1.0)) {
        set_error("cac_server_submit: approx_cut needs a success probability in (0, 1)");
        return CAC_ERR_INVALID;
    }
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->stop) {
        set_error("cac_server_submit: the server is shutting down");
        return CAC_ERR_INVALID;
    }
    r->ticket = s->next_ticket++;
    *ticket = r->ticket;
    Request *raw = r.get();
    s->requests[r->ticket] = std::move(r);
    (req->kind == CAC_QUERY_MINCUT ? s->cut_queue : s->graph_queue).push_back(raw);
    s->cv_work.notify_all();
    return CAC_OK;
}

int cac_server_poll(cac_server *s, uint64_t ticket, int wait, cac_response *resp) {
    if (!s || !resp) {
        set_error("cac_server_poll: invalid argument");
        return CAC_ERR_INVALID;
    }
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->requests.find(ticket);
    if (it == s->requests.end()) {
        set_error("cac_server_poll: unknown ticket " + std::to_string(ticket));
        return CAC_ERR_INVALID;
    }
    Request *r = it->second.get();
    if (!r->done && !wait) return CAC_PENDING;
    s->cv_done.wait(lk, [&] { return r->done; });
    *resp = r->resp;
    s->requests.erase(ticket);
    return CAC_OK;
}

int cac_server_destroy(cac_server *s) {
    if (!s) return CAC_OK;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
        s->cv_work.notify_all();
    }
    if (s->cut_thread.joinable()) s->cut_thread.join();
    if (s->graph_thread.joinable()) s->graph_thread.join();
    cac_ctx_destroy(s->graph);
    cac_ctx_destroy(s->cut);
    cac_ctx_destroy(s->up);
    delete s;
    return CAC_OK;
}

}  // extern "C"
