// tg_serve.cu -- a request loop with continuous batching over one device.
//
// Requests are new meshes (each with a field) and new fields on resident
// meshes.  n_slots worker threads, each with its own CUDA stream, take work
// from one queue: a field request at its head alone, or the new-mesh
// requests near its head that fit the batch size and the device-memory
// budget, merged into one batch (tg_batch_*, the disjoint union).  Requests
// that arrive while the slots are busy therefore join the next batch, and the
// slots' work overlaps on the device.  A finished batch stays resident
// (relations, link adjacency) so later fields on its meshes only classify;
// when memory runs short, idle batches are evicted least-recently-used first
// and a later field on an evicted mesh rebuilds it from the host copy of its
// TV.  A batch whose creation fails (an invalid mesh in it) is retried one
// mesh at a time, so only the invalid request fails.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "tetragpu.h"
#include "tg_internal.h"

namespace {

using Clock = std::chrono::steady_clock;

// device bytes a new mesh is expected to need while it is being processed
// (all relations, the extraction's temporaries, the link adjacency); replaced
// by the measured footprint once its batch is resident
constexpr int64_t kEstBytesPerCell = 800;
constexpr int64_t kEstBytesPerVert = 128;

int64_t estimate(int64_t T, int64_t V) { return kEstBytesPerCell * T + kEstBytesPerVert * V; }

struct Group {                        // a resident batch
    tg_batch *b = nullptr;
    int64_t bytes = 0;
    int64_t live = 0;                 // members not released
    int busy = 0;                     // requests using it now
    uint64_t last_use = 0;
    std::mutex gpu;                   // one thread at a time issues work on it
};

struct MeshRec {
    int64_t id = 0;
    std::vector<int32_t> tv;          // host copy, 4 * T
    int64_t T = 0, V = 0;
    std::shared_ptr<Group> g;         // resident batch, or null (pending / evicted)
    int64_t idx = 0;                  // member index in g
    bool pending = true;              // its first batch has not finished
    bool failed = false;              // its first batch rejected it
    std::mutex build_mu;              // one rebuild at a time after an eviction
};

enum Kind { kMesh = 0, kField = 1 };

struct Req {
    int64_t id = 0;
    Kind kind = kMesh;
    int64_t mesh_id = 0;
    std::shared_ptr<MeshRec> mesh;    // new-mesh requests: the mesh itself
    std::vector<char> field;
    int ftype = TG_FIELD_F32;
    int64_t V = 0;
    Clock::time_point t_submit, t_done;
    bool done = false;
    tg_status status = TG_OK;
    std::string err;
    std::vector<uint32_t> classes;
};

}  // namespace

struct tg_server {
    int device = 0;
    tg_server_config cfg{};
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<std::shared_ptr<Req>> queue;
    std::unordered_map<int64_t, std::shared_ptr<Req>> reqs;
    std::unordered_map<int64_t, std::shared_ptr<MeshRec>> meshes;
    std::vector<std::shared_ptr<Group>> groups;  // resident
    int64_t next_req = 1, next_mesh = 1;
    int64_t used = 0;                 // resident bytes + estimates of work in flight
    int in_flight = 0;
    uint64_t tick = 0;
    bool stop = false;
    tg_server_stats st{};
    std::vector<std::thread> workers;
    std::mutex fg_mu;                 // foreground calls (relation copies)
    cudaStream_t fg = nullptr;
    // one stream per slot; they outlive the workers, because a resident
    // batch's frees are ordered on the stream it was last used on
    std::vector<cudaStream_t> streams;
    // batches dropped under the lock and freed after it is released (a free
    // waits for the batch's last stream, which may be busy with other work)
    std::vector<tg_batch *> graveyard;
};

namespace {

tg_status sfail(tg_status code, const char *msg)
{
    tg::set_last_error(msg);
    return code;
}

void note_used(tg_server *S)
{
    S->st.peak_bytes = std::max(S->st.peak_bytes, S->used);
}

// Free idle resident batches, least recently used first, until `need` bytes
// are released or none is idle.  Called with S->mu held.
void evict_idle(tg_server *S, int64_t need)
{
    std::vector<std::shared_ptr<Group>> idle;
    for (auto &g : S->groups)
        if (g->busy == 0) idle.push_back(g);
    std::sort(idle.begin(), idle.end(),
              [](const std::shared_ptr<Group> &a, const std::shared_ptr<Group> &b) {
                  return a->last_use < b->last_use;
              });
    int64_t freed = 0;
    for (auto &g : idle) {
        if (freed >= need) break;
        for (auto &kv : S->meshes)
            if (kv.second->g == g) kv.second->g.reset();
        S->groups.erase(std::find(S->groups.begin(), S->groups.end(), g));
        S->graveyard.push_back(g->b);
        g->b = nullptr;
        S->used -= g->bytes;
        freed += g->bytes;
        S->st.evictions++;
    }
}

void drop_group_if_unused(tg_server *S, const std::shared_ptr<Group> &g)
{
    if (g->live > 0 || g->busy > 0) return;
    auto it = std::find(S->groups.begin(), S->groups.end(), g);
    if (it == S->groups.end()) return;
    S->groups.erase(it);
    S->graveyard.push_back(g->b);
    g->b = nullptr;
    S->used -= g->bytes;
}

// Free the batches dropped under the lock.  Called without S->mu held.
void bury(tg_server *S)
{
    std::vector<tg_batch *> dead;
    {
        std::lock_guard<std::mutex> lk(S->mu);
        dead.swap(S->graveyard);
    }
    for (tg_batch *b : dead) tg_batch_destroy(b);
}

// Take the next unit of work.  A field request at the head of the queue goes
// alone.  Otherwise the new-mesh requests among the first kScan queued (field
// requests stay where they are) are gathered into one batch, in queue order,
// while they fit the batch size and the memory budget.  A field request is
// never passed by its own mesh's request (that request is ahead of it), so
// moving new meshes forward keeps every field after its mesh.  Called with
// S->mu held; false when the head must wait for memory.
constexpr size_t kScan = 1024;

bool take_work(tg_server *S, std::vector<std::shared_ptr<Req>> &work, int64_t &est)
{
    auto &q = S->queue;
    if (q.front()->kind == kField) {
        work.push_back(q.front());
        q.pop_front();
        est = 0;
        return true;
    }
    const int64_t budget = S->cfg.hbm_budget_bytes;
    int64_t cells = 0;
    est = 0;
    const int ftype = q.front()->ftype;
    std::vector<size_t> pick;
    for (size_t k = 0; k < q.size() && k < kScan; k++) {
        if (q[k]->kind != kMesh || q[k]->ftype != ftype) continue;
        const MeshRec &m = *q[k]->mesh;
        if (!pick.empty() && cells + m.T > S->cfg.batch_cells) break;
        const int64_t e = estimate(m.T, m.V);
        if (S->used + est + e > budget) {
            evict_idle(S, S->used + est + e - budget);
            // nothing in flight will free memory: let a lone request run over
            if (S->used + est + e > budget && !(pick.empty() && S->in_flight == 0)) break;
        }
        est += e;
        cells += m.T;
        pick.push_back(k);
    }
    if (pick.empty()) return false;
    std::deque<std::shared_ptr<Req>> rest;
    size_t next = 0;
    for (size_t k = 0; k < q.size(); k++) {
        if (next < pick.size() && pick[next] == k) {
            work.push_back(q[k]);
            next++;
        } else {
            rest.push_back(q[k]);
        }
    }
    q.swap(rest);
    S->used += est;
    note_used(S);
    return true;
}

// Build one batch from meshes (host TVs), extract, classify their fields.
tg_status build_batch(tg_server *S, const std::vector<std::shared_ptr<MeshRec>> &ms,
                      const std::vector<const char *> &fields, int ftype, cudaStream_t s,
                      tg_batch **out, std::vector<uint32_t> &classes)
{
    const size_t n = ms.size();
    std::vector<int64_t> nc(n), nv(n);
    int64_t T = 0, V = 0;
    for (size_t i = 0; i < n; i++) {
        nc[i] = ms[i]->T;
        nv[i] = ms[i]->V;
        T += nc[i];
        V += nv[i];
    }
    const int32_t *tv = nullptr;
    std::vector<int32_t> cat;
    if (n == 1) {
        tv = ms[0]->tv.data();
    } else {
        cat.resize((size_t)T * 4);
        size_t at = 0;
        for (auto &m : ms) {
            std::memcpy(cat.data() + at, m->tv.data(), m->tv.size() * 4);
            at += m->tv.size();
        }
        tv = cat.data();
    }
    const size_t esz = ftype == TG_FIELD_F64 ? 8 : 4;
    std::vector<char> fcat((size_t)V * esz);
    {
        size_t at = 0;
        for (size_t i = 0; i < n; i++) {
            std::memcpy(fcat.data() + at, fields[i], (size_t)nv[i] * esz);
            at += (size_t)nv[i] * esz;
        }
    }
    tg_batch *b = nullptr;
    tg_status st = tg_batch_create(tv, nc.data(), nv.data(), (int64_t)n, 0, s, &b);
    if (st == TG_OK) st = tg_batch_extract(b, S->cfg.relation_mask | TG_VV, TG_OPT_LINK_ADJACENCY, s);
    classes.assign((size_t)V * 3, 0);
    if (st == TG_OK)
        st = tg_batch_critical_points(b, fcat.data(), ftype, 0, classes.data(), 0, s);
    if (st != TG_OK) {
        if (b) tg_batch_destroy(b);
        return st;
    }
    *out = b;
    return TG_OK;
}

void finish(tg_server *S, const std::shared_ptr<Req> &r, tg_status st, const std::string &err)
{
    r->status = st;
    r->err = err;
    r->t_done = Clock::now();
    r->done = true;
    if (st == TG_OK) S->st.completed++; else S->st.failed++;
}

void run_meshes(tg_server *S, const std::vector<std::shared_ptr<Req>> &work, int64_t est,
                cudaStream_t s)
{
    std::vector<std::shared_ptr<MeshRec>> ms;
    std::vector<const char *> fields;
    {
        std::lock_guard<std::mutex> lk(S->mu);
        for (auto &r : work) {
            ms.push_back(r->mesh);
            fields.push_back(r->field.data());
        }
    }
    const int ftype = work[0]->ftype;
    // one batch; if it fails, each mesh alone (only an invalid mesh fails)
    std::vector<std::vector<size_t>> parts(1);
    for (size_t i = 0; i < work.size(); i++) parts[0].push_back(i);
    std::vector<tg_batch *> built;
    std::vector<std::vector<size_t>> built_parts;
    std::vector<std::vector<uint32_t>> built_classes;
    std::vector<std::pair<size_t, std::pair<tg_status, std::string>>> failed;
    for (size_t p = 0; p < parts.size(); p++) {
        std::vector<std::shared_ptr<MeshRec>> pm;
        std::vector<const char *> pf;
        for (size_t i : parts[p]) {
            pm.push_back(ms[i]);
            pf.push_back(fields[i]);
        }
        tg_batch *b = nullptr;
        std::vector<uint32_t> cls;
        const tg_status st = build_batch(S, pm, pf, ftype, s, &b, cls);
        if (st == TG_OK) {
            built.push_back(b);
            built_parts.push_back(parts[p]);
            built_classes.push_back(std::move(cls));
        } else if (parts[p].size() > 1) {
            const std::vector<size_t> each = parts[p];  // parts grows below
            for (size_t i : each) parts.push_back({i});
        } else {
            failed.push_back({parts[p][0], {st, tg_last_error_string()}});
        }
    }
    std::lock_guard<std::mutex> lk(S->mu);
    S->used -= est;
    S->st.batches += (int64_t)built.size();
    for (size_t k = 0; k < built.size(); k++) {
        auto g = std::make_shared<Group>();
        g->b = built[k];
        g->bytes = tg_mesh_device_bytes(tg_batch_union(built[k]));
        g->last_use = ++S->tick;
        S->used += g->bytes;
        S->groups.push_back(g);
        int64_t v = 0;
        for (size_t j = 0; j < built_parts[k].size(); j++) {
            const size_t i = built_parts[k][j];
            const auto &r = work[i];
            const auto &m = ms[i];
            S->st.meshes_built++;
            auto mit = S->meshes.find(m->id);
            if (mit != S->meshes.end() && mit->second == m) {
                m->g = g;
                m->idx = (int64_t)j;
                g->live++;
            }
            m->pending = false;
            r->classes.assign(built_classes[k].begin() + 3 * v,
                              built_classes[k].begin() + 3 * (v + m->V));
            v += m->V;
            finish(S, r, TG_OK, "");
        }
        drop_group_if_unused(S, g);  // every member released while it ran
    }
    for (auto &f : failed) {
        auto &r = work[f.first];
        finish(S, r, f.second.first, f.second.second);
        ms[f.first]->failed = true;
        ms[f.first]->pending = false;
        S->meshes.erase(r->mesh_id);  // an invalid mesh is not kept
    }
    note_used(S);
    S->in_flight--;
    S->cv_done.notify_all();
    S->cv_work.notify_all();
}

// the resident batch of a mesh, rebuilt alone if it was evicted; busy + 1
tg_status acquire(tg_server *S, int64_t mesh_id, cudaStream_t s, std::shared_ptr<Group> &g,
                  int64_t &idx, int64_t &V)
{
    std::shared_ptr<MeshRec> m;
    auto take = [&]() {
        g = m->g;
        idx = m->idx;
        g->busy++;
        g->last_use = ++S->tick;
    };
    {
        std::unique_lock<std::mutex> lk(S->mu);
        auto it = S->meshes.find(mesh_id);
        if (it == S->meshes.end()) return sfail(TG_ERR_INVALID_ARGUMENT, "unknown or released mesh");
        m = it->second;
        V = m->V;
        // its new-mesh request came first in the queue, so it is in flight
        // (or finished): wait for it rather than building the mesh twice
        S->cv_done.wait(lk, [&] { return !m->pending; });
        if (m->failed) return sfail(TG_ERR_INVALID_MESH, "the mesh was rejected");
        if (m->g) {
            take();
            return TG_OK;
        }
    }
    std::lock_guard<std::mutex> bl(m->build_mu);
    {
        std::lock_guard<std::mutex> lk(S->mu);
        if (m->g) {  // rebuilt by another request meanwhile
            take();
            return TG_OK;
        }
        S->used += estimate(m->T, m->V);
        evict_idle(S, S->used - S->cfg.hbm_budget_bytes);
        note_used(S);
    }
    const int64_t nc = m->T, nv = m->V;
    tg_batch *b = nullptr;
    tg_status st = tg_batch_create(m->tv.data(), &nc, &nv, 1, 0, s, &b);
    if (st == TG_OK) st = tg_batch_extract(b, S->cfg.relation_mask | TG_VV, TG_OPT_LINK_ADJACENCY, s);
    std::lock_guard<std::mutex> lk(S->mu);
    S->used -= estimate(m->T, m->V);
    if (st != TG_OK) {
        if (b) tg_batch_destroy(b);
        return st;
    }
    auto ng = std::make_shared<Group>();
    ng->b = b;
    ng->bytes = tg_mesh_device_bytes(tg_batch_union(b));
    ng->live = S->meshes.count(mesh_id) ? 1 : 0;
    S->used += ng->bytes;
    note_used(S);
    S->groups.push_back(ng);
    S->st.meshes_built++;
    m->g = ng;
    m->idx = 0;
    take();
    return TG_OK;
}

void release_busy(tg_server *S, const std::shared_ptr<Group> &g)
{
    std::lock_guard<std::mutex> lk(S->mu);
    g->busy--;
    drop_group_if_unused(S, g);
}

void run_field(tg_server *S, const std::shared_ptr<Req> &r, cudaStream_t s)
{
    std::shared_ptr<Group> g;
    int64_t idx = 0, V = 0;
    tg_status st = acquire(S, r->mesh_id, s, g, idx, V);
    std::string err;
    if (st == TG_OK) {
        {
            std::lock_guard<std::mutex> gl(g->gpu);
            int64_t v0 = 0;
            st = tg_batch_mesh_offsets(g->b, idx, &v0, nullptr, nullptr, nullptr);
            r->classes.assign((size_t)V * 3, 0);
            if (st == TG_OK)
                st = tg::critical_points_rows(tg_batch_union(g->b), v0, V, r->field.data(),
                                              r->ftype, 0, r->classes.data(), 0, s);
        }
        if (st != TG_OK) err = tg_last_error_string();
        release_busy(S, g);
    } else {
        err = tg_last_error_string();
    }
    std::lock_guard<std::mutex> lk(S->mu);
    finish(S, r, st, err);
    S->in_flight--;
    S->cv_done.notify_all();
    S->cv_work.notify_all();
}

void worker(tg_server *S, cudaStream_t s)
{
    cudaSetDevice(S->device);
    for (;;) {
        std::vector<std::shared_ptr<Req>> work;
        int64_t est = 0;
        {
            std::unique_lock<std::mutex> lk(S->mu);
            for (;;) {
                if (S->queue.empty()) {
                    if (S->stop) return;
                    S->cv_work.wait(lk);
                    continue;
                }
                if (take_work(S, work, est)) break;
                S->cv_work.wait(lk);  // memory frees when work in flight completes
            }
            S->in_flight++;
        }
        bury(S);
        if (work[0]->kind == kField)
            run_field(S, work[0], s);
        else
            run_meshes(S, work, est, s);
        bury(S);
    }
}

}  // namespace

extern "C" {

tg_status tg_server_create(int device, const tg_server_config *cfg, tg_server **out)
{
    if (!out) return sfail(TG_ERR_INVALID_ARGUMENT, "out is NULL");
    *out = nullptr;
    tg_server *S = new tg_server;
    S->device = device;
    if (cfg) S->cfg = *cfg;
    if (S->cfg.n_slots <= 0) S->cfg.n_slots = 4;
    if (S->cfg.hbm_budget_bytes <= 0) S->cfg.hbm_budget_bytes = 150000000000LL;
    if (S->cfg.batch_cells <= 0) S->cfg.batch_cells = 4194304;
    S->cfg.relation_mask &= TG_ALL_RELATIONS;
    int cur = 0;
    cudaGetDevice(&cur);
    cudaError_t e = cudaSetDevice(device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&S->fg, cudaStreamNonBlocking);
    for (int i = 0; e == cudaSuccess && i < S->cfg.n_slots; i++) {
        cudaStream_t st = nullptr;
        e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
        if (e == cudaSuccess) S->streams.push_back(st);
    }
    if (e != cudaSuccess) {
        for (auto st : S->streams) cudaStreamDestroy(st);
        if (S->fg) cudaStreamDestroy(S->fg);
        cudaSetDevice(cur);
        delete S;
        return sfail(TG_ERR_CUDA, cudaGetErrorString(e));
    }
    cudaSetDevice(cur);
    for (int i = 0; i < S->cfg.n_slots; i++) S->workers.emplace_back(worker, S, S->streams[i]);
    *out = S;
    return TG_OK;
}

tg_status tg_server_destroy(tg_server *S)
{
    if (!S) return TG_OK;
    {
        std::lock_guard<std::mutex> lk(S->mu);
        S->stop = true;
    }
    S->cv_work.notify_all();
    for (auto &t : S->workers) t.join();
    bury(S);
    int cur = 0;
    cudaGetDevice(&cur);
    cudaSetDevice(S->device);
    for (auto &g : S->groups) tg_batch_destroy(g->b);
    S->groups.clear();
    for (auto st : S->streams) cudaStreamDestroy(st);
    cudaStreamDestroy(S->fg);
    cudaSetDevice(cur);
    delete S;
    return TG_OK;
}

tg_status tg_server_submit_mesh(tg_server *S, const int32_t *tv, int64_t n_cells, int64_t n_verts,
                                const void *field, int field_type, int64_t *request_id,
                                int64_t *mesh_id)
{
    if (!S || (n_cells > 0 && !tv) || (n_verts > 0 && !field) || n_cells < 0 || n_verts < 0)
        return sfail(TG_ERR_INVALID_ARGUMENT, "bad server, mesh or field");
    if (field_type != TG_FIELD_F32 && field_type != TG_FIELD_F64)
        return sfail(TG_ERR_INVALID_ARGUMENT, "field_type must be TG_FIELD_F32 or TG_FIELD_F64");
    auto m = std::make_shared<MeshRec>();
    m->tv.assign(tv, tv + 4 * n_cells);
    m->T = n_cells;
    m->V = n_verts;
    auto r = std::make_shared<Req>();
    r->kind = kMesh;
    r->mesh = m;
    r->ftype = field_type;
    r->V = n_verts;
    const size_t esz = field_type == TG_FIELD_F64 ? 8 : 4;
    r->field.assign((const char *)field, (const char *)field + esz * n_verts);
    {
        std::lock_guard<std::mutex> lk(S->mu);
        m->id = S->next_mesh++;
        r->id = S->next_req++;
        r->mesh_id = m->id;
        r->t_submit = Clock::now();
        S->meshes[m->id] = m;
        S->reqs[r->id] = r;
        S->queue.push_back(r);
        S->st.submitted++;
    }
    S->cv_work.notify_one();
    if (request_id) *request_id = r->id;
    if (mesh_id) *mesh_id = m->id;
    return TG_OK;
}

tg_status tg_server_submit_field(tg_server *S, int64_t mesh_id, const void *field, int field_type,
                                 int64_t *request_id)
{
    if (!S) return sfail(TG_ERR_INVALID_ARGUMENT, "server is NULL");
    if (field_type != TG_FIELD_F32 && field_type != TG_FIELD_F64)
        return sfail(TG_ERR_INVALID_ARGUMENT, "field_type must be TG_FIELD_F32 or TG_FIELD_F64");
    auto r = std::make_shared<Req>();
    r->kind = kField;
    r->ftype = field_type;
    r->mesh_id = mesh_id;
    {
        std::lock_guard<std::mutex> lk(S->mu);
        auto it = S->meshes.find(mesh_id);
        if (it == S->meshes.end()) return sfail(TG_ERR_INVALID_ARGUMENT, "unknown or released mesh");
        r->V = it->second->V;
        if (r->V > 0 && !field) return sfail(TG_ERR_INVALID_ARGUMENT, "field is NULL");
        const size_t esz = field_type == TG_FIELD_F64 ? 8 : 4;
        r->field.assign((const char *)field, (const char *)field + esz * r->V);
        r->id = S->next_req++;
        r->t_submit = Clock::now();
        S->reqs[r->id] = r;
        S->queue.push_back(r);
        S->st.submitted++;
    }
    S->cv_work.notify_one();
    if (request_id) *request_id = r->id;
    return TG_OK;
}

tg_status tg_server_wait(tg_server *S, int64_t request_id, int64_t timeout_ms,
                         uint32_t *classes_out, double *latency_ms)
{
    if (!S) return sfail(TG_ERR_INVALID_ARGUMENT, "server is NULL");
    std::unique_lock<std::mutex> lk(S->mu);
    auto it = S->reqs.find(request_id);
    if (it == S->reqs.end()) return sfail(TG_ERR_INVALID_ARGUMENT, "unknown request");
    std::shared_ptr<Req> r = it->second;
    if (timeout_ms < 0) {
        S->cv_done.wait(lk, [&] { return r->done; });
    } else if (!S->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms),
                                    [&] { return r->done; })) {
        return sfail(TG_ERR_TIMEOUT, "request not finished");
    }
    S->reqs.erase(request_id);
    if (latency_ms)
        *latency_ms = std::chrono::duration<double, std::milli>(r->t_done - r->t_submit).count();
    if (r->status != TG_OK) return sfail(r->status, r->err.c_str());
    if (classes_out && !r->classes.empty())
        std::memcpy(classes_out, r->classes.data(), r->classes.size() * 4);
    return TG_OK;
}

tg_status tg_server_relation_size(tg_server *S, int64_t mesh_id, int relation, int64_t *rows,
                                  int64_t *entries, int32_t *width)
{
    if (!S || relation < 1 || relation > 13)
        return sfail(TG_ERR_INVALID_ARGUMENT, "bad server or relation");
    std::lock_guard<std::mutex> fg(S->fg_mu);
    int cur = 0;
    cudaGetDevice(&cur);
    cudaSetDevice(S->device);
    std::shared_ptr<Group> g;
    int64_t idx = 0, V = 0;
    tg_status st = acquire(S, mesh_id, S->fg, g, idx, V);
    if (st == TG_OK) {
        {
            std::lock_guard<std::mutex> gl(g->gpu);
            st = tg_batch_extract(g->b, 1u << relation, 0, S->fg);
            if (st == TG_OK) st = tg_batch_relation_size(g->b, idx, relation, rows, entries, width);
        }
        release_busy(S, g);
    }
    bury(S);
    cudaSetDevice(cur);
    return st;
}

tg_status tg_server_copy_relation(tg_server *S, int64_t mesh_id, int relation,
                                  int64_t *offsets_out, int32_t *entries_out)
{
    if (!S || relation < 1 || relation > 13)
        return sfail(TG_ERR_INVALID_ARGUMENT, "bad server or relation");
    std::lock_guard<std::mutex> fg(S->fg_mu);
    int cur = 0;
    cudaGetDevice(&cur);
    cudaSetDevice(S->device);
    std::shared_ptr<Group> g;
    int64_t idx = 0, V = 0;
    tg_status st = acquire(S, mesh_id, S->fg, g, idx, V);
    if (st == TG_OK) {
        {
            std::lock_guard<std::mutex> gl(g->gpu);
            st = tg_batch_extract(g->b, 1u << relation, 0, S->fg);
            if (st == TG_OK)
                st = tg_batch_copy_relation(g->b, idx, relation, offsets_out, entries_out, S->fg);
        }
        release_busy(S, g);
    }
    bury(S);
    cudaSetDevice(cur);
    return st;
}

tg_status tg_server_release_mesh(tg_server *S, int64_t mesh_id)
{
    if (!S) return sfail(TG_ERR_INVALID_ARGUMENT, "server is NULL");
    {
        std::lock_guard<std::mutex> lk(S->mu);
        auto it = S->meshes.find(mesh_id);
        if (it == S->meshes.end())
            return sfail(TG_ERR_INVALID_ARGUMENT, "unknown or released mesh");
        std::shared_ptr<Group> g = it->second->g;
        S->meshes.erase(it);
        if (g) {
            g->live--;
            drop_group_if_unused(S, g);
        }
    }
    bury(S);
    return TG_OK;
}

tg_status tg_server_get_stats(tg_server *S, tg_server_stats *out)
{
    if (!S || !out) return sfail(TG_ERR_INVALID_ARGUMENT, "NULL argument");
    std::lock_guard<std::mutex> lk(S->mu);
    *out = S->st;
    out->resident_meshes = 0;
    out->resident_bytes = 0;
    for (auto &g : S->groups) {
        out->resident_meshes += g->live;
        out->resident_bytes += g->bytes;
    }
    return TG_OK;
}

}  // extern "C"
