// batch.cu -- many independent HFB instances of uneven size run concurrently.
//
// The reference runs one nucleus per process (src/Main.f90); a batch drives
// many contexts -- each with its own mesh, spwf count, particle numbers and
// constraints, each on its own streams -- from a pool of host worker threads,
// so that the latency-bound parts of one instance (the Fermi search of the
// pairing step reads its particle numbers back, small eigenproblems, the
// Coulomb solve) overlap with the mesh kernels of others on the 152 SMs.
//
// Schedule: each worker owns a list of instances and runs them round-robin,
// one Evolve pass each per round.  The lists come from a longest-first (LPT)
// assignment of the instances' measured iteration times.  mg_batch_tune is
// the autotuner: it times one pass of every instance alone, then a few
// rounds for each candidate worker count, and keeps the fastest.
#include <algorithm>
#include <chrono>
#include <numeric>
#include <thread>
#include <vector>

#include "mg_internal.cuh"

struct mg_batch {
    std::vector<mg_ctx*> ctx;
    std::vector<double> cost;                // seconds per Evolve pass (measured, or a model)
    std::vector<std::vector<int>> lists;     // per worker: instance indices
    std::vector<int> status;                 // per instance: last status (< 0: failed, skipped)
    int device = 0;
    int workers = 1;
};

namespace {

double now_s() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch())
        .count();
}

// Longest processing time first: instances by decreasing cost, each to the
// least-loaded worker.
void assign(mg_batch* b, int workers) {
    const int n = (int)b->ctx.size();
    workers = std::max(1, std::min(workers, n));
    std::vector<int> order(n);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(),
                     [&](int x, int y) { return b->cost[x] > b->cost[y]; });
    b->lists.assign(workers, {});
    std::vector<double> load(workers, 0.0);
    for (int i : order) {
        const int w = (int)(std::min_element(load.begin(), load.end()) - load.begin());
        b->lists[w].push_back(i);
        load[w] += b->cost[i];
    }
    b->workers = workers;
}

int run(mg_batch* b, int n_iter, const double* dt, const double* mom, mg_energy_terms* out) {
    const int W = (int)b->lists.size();
    std::vector<int> status(W, MG_OK);
    // An instance whose pass fails (negative status) is marked failed and
    // skipped from then on; the others carry on.  A worker reports the first
    // failure it saw, else the largest positive status.
    auto work = [&](int w) {
        if (cudaSetDevice(b->device) != cudaSuccess) { status[w] = MG_ERR_CUDA; return; }
        int st = MG_OK;
        for (int k = 0; k < n_iter; ++k)
            for (int i : b->lists[w]) {
                if (b->status[i] < 0) continue;
                const int s = mg_iterate(b->ctx[i], 1, dt[i], mom[i], out ? &out[i] : nullptr);
                b->status[i] = s;
                if (s < 0) { if (st >= 0) st = s; continue; }
                if (st >= 0) st = std::max(st, s);
            }
        // every instance's work is complete when the call returns
        for (int i : b->lists[w]) {
            if (b->status[i] < 0) continue;
            const int s = mg_synchronize(b->ctx[i]);
            if (s < 0) {
                b->status[i] = s;
                if (st >= 0) st = s;
            }
        }
        status[w] = st;
    };
    if (W == 1) {
        work(0);
    } else {
        std::vector<std::thread> th;
        th.reserve(W);
        for (int w = 0; w < W; ++w) th.emplace_back(work, w);
        for (std::thread& t : th) t.join();
    }
    int st = MG_OK;
    for (int s : status) {
        if (s < 0) return s;
        st = std::max(st, s);
    }
    return st;
}

}  // namespace

extern "C" int mg_batch_create(int n, mg_ctx* const* ctxs, mg_batch** out) {
    if (!out) return MG_ERR_ARG;
    *out = nullptr;
    if (n <= 0 || !ctxs) return MG_ERR_ARG;
    for (int i = 0; i < n; ++i)
        if (!ctxs[i]) return MG_ERR_ARG;
    // one entry per context: two workers must never run the same context
    std::vector<mg_ctx*> sorted(ctxs, ctxs + n);
    std::sort(sorted.begin(), sorted.end());
    if (std::adjacent_find(sorted.begin(), sorted.end()) != sorted.end()) return MG_ERR_ARG;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return MG_ERR_CUDA;
    for (int i = 0; i < n; ++i)
        if (ctxs[i]->device != dev) return MG_ERR_ARG;   // all on the current device
    mg_batch* b = new mg_batch();
    b->ctx.assign(ctxs, ctxs + n);
    // cost model until measured: mesh work ~ nwt V per basis
    for (mg_ctx* c : b->ctx)
        b->cost.push_back((double)c->p.nwt * (double)c->V * (c->p.pairing == MG_PAIRING_HFB ? 2 : 1));
    b->status.assign(n, MG_OK);
    b->device = dev;
    const int hw = (int)std::max(1u, std::thread::hardware_concurrency());
    assign(b, std::min(n, hw));
    *out = b;
    return MG_OK;
}

extern "C" int mg_batch_destroy(mg_batch* b) {
    delete b;
    return MG_OK;
}

extern "C" int mg_batch_status(mg_batch* b, int* status) {
    if (!b || !status) return MG_ERR_ARG;
    for (size_t i = 0; i < b->status.size(); ++i) status[i] = b->status[i];
    return MG_OK;
}

extern "C" int mg_batch_set_workers(mg_batch* b, int workers) {
    if (!b || workers <= 0) return MG_ERR_ARG;
    assign(b, workers);
    return b->workers;
}

extern "C" int mg_batch_iterate(mg_batch* b, int n_iter, const double* dt, const double* momentum,
                                mg_energy_terms* out) {
    if (!b || n_iter < 0 || !dt || !momentum) return MG_ERR_ARG;
    return run(b, n_iter, dt, momentum, out);
}

extern "C" int mg_batch_tune(mg_batch* b, int probe, const double* dt, const double* momentum,
                             int* workers_out) {
    if (!b || probe <= 0 || !dt || !momentum) return MG_ERR_ARG;
    const int n = (int)b->ctx.size();
    // 1. each instance alone: its iteration time (this also makes every
    //    allocation an instance does lazily on its first passes)
    int first_err = MG_OK;
    for (int i = 0; i < n; ++i) {
        double best = 1e30;
        for (int k = 0; k < probe && b->status[i] >= 0; ++k) {
            const double t0 = now_s();
            int s = mg_iterate(b->ctx[i], 1, dt[i], momentum[i], nullptr);
            if (s >= 0) {
                const int s2 = mg_synchronize(b->ctx[i]);
                if (s2 < 0) s = s2;
            }
            b->status[i] = s;
            if (s < 0 && first_err == MG_OK) first_err = s;
            best = std::min(best, now_s() - t0);
        }
        b->cost[i] = best;
    }
    // 2. candidate worker counts, `probe` rounds each
    const int hw = (int)std::max(1u, std::thread::hardware_concurrency());
    std::vector<int> cand;
    for (int w = 1; w <= std::min(n, 4 * hw); w *= 2) cand.push_back(w);
    if (n <= 4 * hw && (cand.empty() || cand.back() != n)) cand.push_back(n);
    double best_t = 1e30;
    int best_w = 1;
    for (int w : cand) {
        assign(b, w);
        const double t0 = now_s();
        const int s = run(b, probe, dt, momentum, nullptr);
        if (s < 0 && first_err == MG_OK) first_err = s;
        const double t = now_s() - t0;
        if (t < best_t) { best_t = t; best_w = b->workers; }
    }
    assign(b, best_w);
    if (workers_out) *workers_out = best_w;
    return first_err;
}
