// Continuous-batching lensing server in the library (the host scheduler of the
// served form).  The reference has no serving layer: its transformers process
// one call at a time with device-wide synchronisation
// (cunusht/helper_GPU.py:27-51).
//
// Requests -- lensing (gclm -> lensed map, gclm2lenmap) or delensing (lensed
// map -> gclm, lenmap2gclm) of any lmax, spin and accuracy on a Gauss-Legendre
// pointing grid -- are queued per bucket (lmax, spin, eps, nphi).  A bucket
// owns slots; a slot is a plan with its batch workspace, static input / output
// buffers and its own CUDA stream, and runs at most one launch at a time.
// cunusht_server_poll() retires launches whose events have completed and
// fills every idle slot with the requests waiting in its bucket, so requests
// that arrive while others run are admitted as soon as a slot frees up, and
// launches of different slots overlap on the device.  A launch copies the
// requests' inputs into the slot's static buffers, replays the CUDA graph of
// the batched entry point (captured on first use per direction and batch
// size) and copies the results to the caller's output buffers, all on the
// slot's stream.  A bucket's slots are created only if the device memory they
// take (measured with cudaMemGetInfo) fits the HBM budget; idle buckets are
// released to make room.
#include <algorithm>
#include <cmath>
#include <deque>
#include <map>
#include <memory>
#include <set>
#include <tuple>
#include <vector>

#include "common.cuh"
#include "kernels.cuh"

using namespace cunusht;

namespace {

struct Req {
    int64_t id;
    int dir;  // 0 lensing, 1 delensing
    const void *in;
    const void *dlm;
    void *out;
    cudaEvent_t ready;  // recorded on the caller's stream at submission (or NULL)
};

struct Slot {
    cunusht_plan_t *plan = nullptr;
    cudaStream_t st = nullptr;
    cudaEvent_t ev = nullptr;
    int spin = 0, ncomp = 1, cap = 1;
    long long npix = 0, nalm = 0;
    double2 *gin = nullptr, *din = nullptr, *aout = nullptr;
    double *mout = nullptr, *lin = nullptr;
    std::map<std::pair<int, int>, cudaGraphExec_t> graphs;  // (direction, batch size)
    std::vector<Req> busy;
    size_t bytes = 0;

    ~Slot() {
        for (auto &g : graphs) cudaGraphExecDestroy(g.second);
        void *bufs[] = {gin, din, mout};  // aout, lin alias gin, mout
        for (void *b : bufs)
            if (b) cudaFree(b);
        if (ev) cudaEventDestroy(ev);
        if (st) cudaStreamDestroy(st);
        if (plan) cunusht_plan_destroy(plan);
    }
};

using Key = std::tuple<int, int, double, int>;  // lmax, spin, eps, nphi

struct Bucket {
    std::vector<std::unique_ptr<Slot>> slots;
};

}  // namespace

struct cunusht_server_s {
    double budget = 150e9;
    int precision = CUNUSHT_PREC_MIXED;
    std::map<int, std::pair<int, int>> policy;  // lmax -> (requests per launch, slots)
    std::map<Key, Bucket> buckets;
    std::map<Key, std::deque<Req>> queues;
    std::map<Key, size_t> sizes;       // measured device bytes of each bucket's slots
    std::map<Key, long long> last_use;  // launch counter at each bucket's last launch
    std::set<Key> refused;              // buckets waiting for room
    std::vector<int64_t> done;
    int64_t next_id = 1;
    long long launches = 0, completed = 0, refusals = 0, evictions = 0;

    size_t used() const {
        size_t u = 0;
        for (auto &b : buckets)
            for (auto &s : b.second.slots) u += s->bytes;
        return u;
    }
    std::pair<int, int> policy_of(int lmax) const {
        auto it = policy.find(lmax);
        if (it != policy.end()) return it->second;
        return lmax >= 4095 ? std::make_pair(1, 1) : (lmax >= 2047 ? std::make_pair(4, 2) : std::make_pair(8, 2));
    }
};

namespace {

size_t free_bytes() {
    size_t f = 0, t = 0;
    cudaMemGetInfo(&f, &t);
    return f;
}

// Stream priority of a bucket's slots: the smaller the transform, the higher
// the priority, so that a short launch takes the SMs that free up while long
// launches of larger lmax are resident instead of waiting behind their
// thousands of blocks (lmax <= 1023: highest, 2047: one below, larger: the
// default).
int slot_priority(int lmax) {
    int least = 0, greatest = 0;
    if (cudaDeviceGetStreamPriorityRange(&least, &greatest) != cudaSuccess) return 0;
    const int rank = lmax <= 1023 ? 2 : lmax <= 2047 ? 1 : 0;  // levels above the default
    return std::max(greatest, least - rank);
}

// GL pointing geometry with nphi pixels per ring (geometry.py:267-284)
int make_slot(cunusht_server_s *S, const Key &k, int cap, std::unique_ptr<Slot> &out) {
    const int lmax = std::get<0>(k), spin = std::get<1>(k), nphi = std::get<3>(k);
    const double eps = std::get<2>(k);
    CU_TRY(cudaDeviceSynchronize());
    const size_t f0 = free_bytes();
    auto sl = std::make_unique<Slot>();
    const int nring = lmax + 1;
    std::vector<double> x, w, th(nring), p0(nring, 0.0);
    gauss_legendre(nring, x, w);
    for (int r = 0; r < nring; ++r) th[r] = std::acos(x[r]);
    std::sort(th.begin(), th.end());
    std::vector<int64_t> nph(nring, nphi), ofs(nring);
    for (int r = 0; r < nring; ++r) ofs[r] = (int64_t)r * nphi;
    RC_TRY(cunusht_plan_create(&sl->plan, lmax, eps, S->precision, std::max(spin, 1), nring, th.data(), p0.data(),
                               nph.data(), ofs.data()));
    RC_TRY(cunusht_plan_reserve_batch(sl->plan, cap));
    if (sl->plan->prec == CUNUSHT_PREC_MIXED) {
        // the batched solves read the start states of the CC grid at the bucket's
        // spin and of the pointing grid at spin 1 only
        for (int s = 0; s <= std::max(spin, 1); ++s) {
            if (s != 1) RC_TRY(cunusht_plan_set_start_states(sl->plan, 0, s, 0));
            if (s != spin) RC_TRY(cunusht_plan_set_start_states(sl->plan, 1, s, 0));
        }
    }
    sl->spin = spin;
    sl->ncomp = spin ? 2 : 1;
    sl->cap = cap;
    sl->npix = (long long)nring * nphi;
    sl->nalm = (long long)(lmax + 1) * (lmax + 2) / 2;
    const long long ncm = spin ? 2 : 1;
    CU_TRY(cudaMalloc(&sl->gin, sizeof(double2) * cap * sl->ncomp * sl->nalm));
    CU_TRY(cudaMalloc(&sl->din, sizeof(double2) * cap * sl->nalm));
    CU_TRY(cudaMalloc(&sl->mout, sizeof(double) * cap * ncm * sl->npix));
    // a launch runs one direction: the delensing maps in share the lensing maps
    // out, the delensing alm out the lensing alm in
    sl->lin = sl->mout;
    sl->aout = sl->gin;
    // zeroed inputs: a prewarm run (graph capture ahead of traffic) reads them
    CU_TRY(cudaMemset(sl->gin, 0, sizeof(double2) * cap * sl->ncomp * sl->nalm));
    CU_TRY(cudaMemset(sl->din, 0, sizeof(double2) * cap * sl->nalm));
    CU_TRY(cudaMemset(sl->lin, 0, sizeof(double) * cap * ncm * sl->npix));
    CU_TRY(cudaStreamCreateWithPriority(&sl->st, cudaStreamNonBlocking, slot_priority(lmax)));
    CU_TRY(cudaEventCreateWithFlags(&sl->ev, cudaEventDisableTiming));
    CU_TRY(cudaDeviceSynchronize());
    const size_t f1 = free_bytes();
    sl->bytes = f0 > f1 ? f0 - f1 : 0;
    out = std::move(sl);
    return CUNUSHT_OK;
}

int run_batch(Slot *sl, int dir, int n) {
    if (dir == 0)
        return cunusht_lensing_batch(sl->plan, n, sl->spin, sl->ncomp, sl->gin, sl->din, nullptr, nullptr, nullptr,
                                     sl->mout, CUNUSHT_F64, sl->st);
    return cunusht_delensing_batch(sl->plan, n, sl->spin, sl->ncomp, sl->lin, CUNUSHT_F64, sl->din, nullptr, nullptr,
                                   nullptr, sl->aout, sl->st);
}

// capture the (direction, n) graph of a slot if it has none yet
int capture_graph(Slot *sl, int dir, int n) {
    auto key = std::make_pair(dir, n);
    if (sl->graphs.count(key)) return CUNUSHT_OK;
    RC_TRY(run_batch(sl, dir, n));  // eager first run: kernel attributes, module loading
    cudaGraph_t g = nullptr;
    CU_TRY(cudaStreamBeginCapture(sl->st, cudaStreamCaptureModeThreadLocal));
    const int rc = run_batch(sl, dir, n);
    const cudaError_t e = cudaStreamEndCapture(sl->st, &g);
    if (rc != CUNUSHT_OK) {
        if (g) cudaGraphDestroy(g);
        return rc;
    }
    CU_TRY(e);
    cudaGraphExec_t ex = nullptr;
    const cudaError_t ei = cudaGraphInstantiate(&ex, g, 0);
    cudaGraphDestroy(g);
    CU_TRY(ei);
    sl->graphs.emplace(key, ex);
    return CUNUSHT_OK;
}

// replay the (direction, n) graph, capturing it on first use
int launch_graph(Slot *sl, int dir, int n) {
    RC_TRY(capture_graph(sl, dir, n));
    CU_TRY(cudaGraphLaunch(sl->graphs.at(std::make_pair(dir, n)), sl->st));
    return CUNUSHT_OK;
}

int launch(cunusht_server_s *S, Slot *sl, std::deque<Req> &q) {
    const int dir = q.front().dir;
    std::vector<Req> batch;
    while (!q.empty() && q.front().dir == dir && (int)batch.size() < sl->cap) {
        batch.push_back(q.front());
        q.pop_front();
    }
    const int n = (int)batch.size();
    const long long ncm = sl->spin ? 2 : 1;
    const size_t abytes = sizeof(double2) * sl->ncomp * sl->nalm, mbytes = sizeof(double) * ncm * sl->npix;
    for (int i = 0; i < n; ++i) {
        Req &r = batch[i];
        if (r.ready) {  // inputs written on the caller's stream
            CU_TRY(cudaStreamWaitEvent(sl->st, r.ready, 0));
            cudaEventDestroy(r.ready);
            r.ready = nullptr;
        }
        if (dir == 0)
            CU_TRY(cudaMemcpyAsync((char *)sl->gin + i * abytes, r.in, abytes, cudaMemcpyDeviceToDevice, sl->st));
        else
            CU_TRY(cudaMemcpyAsync((char *)sl->lin + i * mbytes, r.in, mbytes, cudaMemcpyDeviceToDevice, sl->st));
        CU_TRY(cudaMemcpyAsync(sl->din + i * sl->nalm, r.dlm, sizeof(double2) * sl->nalm, cudaMemcpyDeviceToDevice,
                               sl->st));
    }
    RC_TRY(launch_graph(sl, dir, n));
    for (int i = 0; i < n; ++i) {
        const Req &r = batch[i];
        if (dir == 0)
            CU_TRY(cudaMemcpyAsync(r.out, (char *)sl->mout + i * mbytes, mbytes, cudaMemcpyDeviceToDevice, sl->st));
        else
            CU_TRY(cudaMemcpyAsync(r.out, (char *)sl->aout + i * abytes, abytes, cudaMemcpyDeviceToDevice, sl->st));
    }
    CU_TRY(cudaEventRecord(sl->ev, sl->st));
    sl->busy = std::move(batch);
    S->launches += 1;
    return CUNUSHT_OK;
}

// Release idle buckets other than keep (empty queue, nothing in flight),
// least recently used first, until at least free bytes are released; release
// nothing and return false if all the idle buckets together hold less.
bool release_lru(cunusht_server_s *S, const Key &keep, size_t free) {
    std::vector<std::pair<long long, Key>> idle;
    for (auto &b : S->buckets) {
        if (b.first == keep || !S->queues[b.first].empty()) continue;
        bool busy = false;
        for (auto &s : b.second.slots) busy = busy || !s->busy.empty();
        if (!busy) idle.emplace_back(S->last_use[b.first], b.first);
    }
    std::sort(idle.begin(), idle.end());
    std::vector<Key> chosen;
    size_t got = 0;
    for (auto &c : idle) {
        if (got >= free) break;
        chosen.push_back(c.second);
        for (auto &s : S->buckets[c.second].slots) got += s->bytes;
    }
    if (got < free) return false;
    for (auto &k : chosen) {
        S->buckets.erase(k);
        S->evictions += 1;
    }
    return true;
}

void refuse(cunusht_server_s *S, const Key &k) {
    if (S->refused.insert(k).second) S->refusals += 1;  // one count per refused episode
}

// Slots for bucket k within the budget.  Once a bucket's size is known
// (measured when its slots were first made), a bucket that does not fit
// releases idle buckets, least recently used first and only as many as it
// needs, or none when all the idle ones together would not make room, and
// waits; the size check comes before any allocation.  evict = false
// (prewarm) releases nothing.
int admit(cunusht_server_s *S, const Key &k, bool &ok, bool evict = true) {
    ok = S->buckets.count(k) > 0;
    if (ok) return CUNUSHT_OK;
    size_t used = S->used();
    auto sz = S->sizes.find(k);
    if (sz != S->sizes.end() && (double)(used + sz->second) > S->budget) {
        const size_t free = (size_t)((double)(used + sz->second) - S->budget) + 1;
        if (!evict || !release_lru(S, k, free)) {
            refuse(S, k);
            return CUNUSHT_OK;
        }
        used = S->used();
    }
    const auto pol = S->policy_of(std::get<0>(k));
    Bucket b;
    size_t add = 0;
    for (int i = 0; i < pol.second; ++i) {
        std::unique_ptr<Slot> sl;
        if (make_slot(S, k, pol.first, sl) != CUNUSHT_OK) {
            cudaGetLastError();  // an allocation failure is a refusal, not an error
            break;
        }
        if ((double)(used + add + sl->bytes) > S->budget) {
            S->sizes[k] = (size_t)pol.second * sl->bytes;  // known for the next attempt
            break;
        }
        add += sl->bytes;
        b.slots.push_back(std::move(sl));
    }
    if (b.slots.empty()) {
        refuse(S, k);
        return CUNUSHT_OK;
    }
    S->refused.erase(k);
    S->sizes[k] = add;
    S->last_use[k] = S->launches;
    S->buckets.emplace(k, std::move(b));
    ok = true;
    return CUNUSHT_OK;
}

}  // namespace

extern "C" {

int cunusht_server_create(cunusht_server_t **srv, double hbm_budget_bytes, int precision) {
    clear_error();
    ARG_CHECK(srv != nullptr, "server output pointer is NULL");
    ARG_CHECK(hbm_budget_bytes > 0, "HBM budget must be positive");
    ARG_CHECK(precision >= 0 && precision <= 2, "precision must be 0 (auto), 1 (fp64) or 2 (mixed)");
    auto *S = new cunusht_server_s();
    S->budget = hbm_budget_bytes;
    S->precision = precision;
    *srv = S;
    return CUNUSHT_OK;
}

int cunusht_server_set_policy(cunusht_server_t *S, int lmax, int requests_per_launch, int slots) {
    clear_error();
    ARG_CHECK(S != nullptr, "server is NULL");
    ARG_CHECK(requests_per_launch >= 1 && requests_per_launch <= 64 && slots >= 1 && slots <= 8,
              "requests per launch must be in [1, 64] and slots in [1, 8]");
    S->policy[lmax] = std::make_pair(requests_per_launch, slots);
    return CUNUSHT_OK;
}

int cunusht_server_submit(cunusht_server_t *S, int direction, int lmax, int spin, double eps, int nphi,
                          const void *input, const void *dlm_scaled, void *output, void *producer_stream,
                          int64_t *request_id) {
    clear_error();
    ARG_CHECK(S != nullptr, "server is NULL");
    ARG_CHECK(direction == 0 || direction == 1, "direction must be 0 (lensing) or 1 (delensing)");
    ARG_CHECK(lmax >= 1 && lmax <= 4095, "lmax must be in [1, 4095], got %d", lmax);
    ARG_CHECK(spin >= 0 && spin <= 2, "spin must be 0, 1 or 2");
    ARG_CHECK(input && dlm_scaled && output, "NULL array argument");
    if (nphi <= 0) nphi = 2 * lmax + 1;
    const Key k(lmax, spin, eps, nphi);
    Req r{S->next_id++, direction, input, dlm_scaled, output, nullptr};
    CU_TRY(cudaEventCreateWithFlags(&r.ready, cudaEventDisableTiming));
    CU_TRY(cudaEventRecord(r.ready, (cudaStream_t)producer_stream));
    S->queues[k].push_back(r);
    if (request_id) *request_id = r.id;
    return CUNUSHT_OK;
}

int cunusht_server_poll(cunusht_server_t *S, int64_t *done_ids, int max_ids, int *ndone, int *pending) {
    clear_error();
    ARG_CHECK(S != nullptr, "server is NULL");
    // retire
    for (auto &b : S->buckets)
        for (auto &sl : b.second.slots) {
            if (sl->busy.empty()) continue;
            const cudaError_t e = cudaEventQuery(sl->ev);
            if (e == cudaErrorNotReady) continue;
            CU_TRY(e);
            for (auto &r : sl->busy) S->done.push_back(r.id);
            S->completed += (long long)sl->busy.size();
            sl->busy.clear();
        }
    // admit and launch
    int npend = 0;
    for (auto &kq : S->queues) {
        auto &q = kq.second;
        if (q.empty()) continue;
        bool ok = false;
        RC_TRY(admit(S, kq.first, ok));
        if (!ok) continue;
        for (auto &sl : S->buckets[kq.first].slots)
            if (!q.empty() && sl->busy.empty()) {
                RC_TRY(launch(S, sl.get(), q));
                S->last_use[kq.first] = S->launches;
            }
    }
    for (auto &kq : S->queues) npend += (int)kq.second.size();
    for (auto &b : S->buckets)
        for (auto &sl : b.second.slots) npend += (int)sl->busy.size();
    int n = 0;
    if (done_ids && max_ids > 0) {
        n = std::min<int>(max_ids, (int)S->done.size());
        std::copy(S->done.begin(), S->done.begin() + n, done_ids);
        S->done.erase(S->done.begin(), S->done.begin() + n);
    }
    if (ndone) *ndone = n;
    if (pending) *pending = npend;
    return CUNUSHT_OK;
}

int cunusht_server_stats(cunusht_server_t *S, double *stats, int n) {
    clear_error();
    ARG_CHECK(S != nullptr && stats != nullptr, "NULL argument");
    int nslots = 0;
    for (auto &b : S->buckets) nslots += (int)b.second.slots.size();
    const double v[7] = {(double)S->launches, (double)S->completed, (double)S->used(), (double)S->buckets.size(),
                         (double)nslots, (double)S->refusals, (double)S->evictions};
    for (int i = 0; i < n && i < 7; ++i) stats[i] = v[i];
    return CUNUSHT_OK;
}

int cunusht_server_prewarm(cunusht_server_t *S, int lmax, int spin, double eps, int nphi, int *admitted) {
    clear_error();
    ARG_CHECK(S != nullptr, "server is NULL");
    ARG_CHECK(lmax >= 1 && lmax <= 4095, "lmax must be in [1, 4095], got %d", lmax);
    ARG_CHECK(spin >= 0 && spin <= 2, "spin must be 0, 1 or 2");
    if (nphi <= 0) nphi = 2 * lmax + 1;
    const Key k(lmax, spin, eps, nphi);
    bool ok = false;
    RC_TRY(admit(S, k, ok, false));
    if (admitted) *admitted = ok ? 1 : 0;
    if (!ok) return CUNUSHT_OK;
    for (auto &sl : S->buckets[k].slots) {
        if (!sl->busy.empty()) continue;  // a slot with work in flight keeps capturing lazily
        for (int dir = 0; dir < 2; ++dir)
            for (int n = 1; n <= sl->cap; ++n) RC_TRY(capture_graph(sl.get(), dir, n));
    }
    CU_TRY(cudaDeviceSynchronize());
    return CUNUSHT_OK;
}

int cunusht_server_destroy(cunusht_server_t *S) {
    clear_error();
    if (!S) return CUNUSHT_OK;
    cudaDeviceSynchronize();
    for (auto &kq : S->queues)
        for (auto &r : kq.second)
            if (r.ready) cudaEventDestroy(r.ready);
    delete S;
    return CUNUSHT_OK;
}

}  // extern "C"
