/*
 * J for a batch of structures (molecules of uneven size) in shared launches.
 *
 * The reference's callers build one J at a time (H2P-ERI
 * tests/test_J_input_mat.c:46-50); a batch of small and large molecules then
 * runs one chain of ~20 dependent launches per molecule, most of them too
 * small to fill the GPU. Here the 128 x 128 tiles of the tensor-core plan of
 * every structure are merged phase by phase into one batch plan:
 *   near field, stages 1..3   (all lanes of every structure)
 *   upward sweep, level k     (k-th level from the leaves of each structure)
 *   coupling, stages 1..3
 *   downward sweep, level k   (k-th level from the top of each structure)
 * Each structure keeps its own order of phases, so its dependencies hold,
 * while every launch carries the tiles of all structures: about 18 launches
 * of the multi-density kernel for the whole batch. Where the structures'
 * launch choices (default or tuned) put their density count on the
 * single-density kernels instead, the same merge is made of their tile
 * plans for the mixed single-density kernel (near-field stages split by
 * storage format). Each tile names its
 * structure (vector spaces and number of densities in a small table) and
 * carries the device address of its slices. The plan is built once for a
 * set of structures and their densities per structure, and reused while
 * they and their work buffers stay the same.
 */
#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "h2eri_gb300.h"
#include "h2g_gpu_api.h"

namespace h2g {

#define BCUDA_TRY(call)                                                                          \
    do {                                                                                         \
        cudaError_t e_ = (call);                                                                 \
        if (e_ != cudaSuccess) {                                                                 \
            set_error(std::string(#call) + ": " + cudaGetErrorString(e_));                      \
            return 10;                                                                           \
        }                                                                                        \
    } while (0)

namespace {

struct BatchPlan {
    bool simt = false;                  /* single-density tile kernel (else the tensor-core kernel) */
    std::vector<const DevRep *> reps;
    std::vector<int> n_den;
    std::vector<const void *> bufs;     /* x, y and work buffers each plan entry points at */
    std::vector<const void *> plans;    /* the structures' tile lists the plan was made from */
    TileM *tiles = nullptr;             /* tensor-core plan */
    int8_t *scales = nullptr;
    Tile *stiles = nullptr;             /* single-density plan: tiles and concatenated tensor maps */
    void *maps = nullptr;
    BatchMol *mols = nullptr;
    std::vector<Range> phases;          /* launch order (pair: float-pair format, single-density plan) */
    int nf_phases = 0;                  /* the first nf_phases are the near field (own stream) */
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    int n_tiles = 0;
    ~BatchPlan()
    {
        if (ev_fork) cudaEventDestroy(ev_fork);
        if (ev_join) cudaEventDestroy(ev_join);
        cudaFree(tiles);
        cudaFree(scales);
        cudaFree(stiles);
        cudaFree(maps);
        cudaFree(mols);
    }
};

std::mutex g_bmu;
BatchPlan *g_bplan = nullptr;   /* the last batch plan (one batch at a time is the use case) */

VecArgs rep_vecargs(const DevRep *d, int nvec)
{
    VecArgs va;
    std::memset(&va, 0, sizeof(va));
    const size_t per_r = (size_t)d->rank_total * nvec;
    va.base[VK_X] = d->xbuf;
    va.stride[VK_X] = d->krnl;
    va.base[VK_Y] = d->ybuf;
    va.stride[VK_Y] = d->krnl;
    va.base[VK_Y0] = d->work;
    va.stride[VK_Y0] = d->rank_total;
    va.base[VK_Y1] = d->work + per_r;
    va.stride[VK_Y1] = d->rank_total;
    va.base[VK_T] = d->work + 2 * per_r;
    va.stride[VK_T] = d->lr_total;
    return va;
}

bool same_plan(const BatchPlan *p, bool simt, int n, DevRep *const *reps, const int *n_den)
{
    if (p == nullptr || p->simt != simt || (int)p->reps.size() != n) return false;
    for (int i = 0; i < n; i++)
        if (p->reps[i] != reps[i] || p->n_den[i] != n_den[i] || p->bufs[3 * i] != reps[i]->xbuf ||
            p->bufs[3 * i + 1] != reps[i]->ybuf || p->bufs[3 * i + 2] != reps[i]->work ||
            p->plans[i] != (const void *)reps[i]->tiles)
            return false;
    return true;
}

/* The single-density batch plan: phases near field stage s (float pairs,
 * then single floats), upward levels, coupling stages, downward levels,
 * each with the tiles of every structure; tensor-map indices shifted into
 * the concatenated map array, the structure index in Tile::a. */
int build_plan_simt(int n, DevRep *const *reps, const int *n_den, BatchPlan *p)
{
    std::vector<Tile> all;
    std::vector<int> map_off(n, 0);
    size_t n_maps = 0;
    for (int i = 0; i < n; i++) {
        map_off[i] = (int)n_maps;
        n_maps += std::max<size_t>(reps[i]->mixed_items.size(), 1);
    }
    auto merge = [&](bool pair, auto pick) {
        Range r;
        r.first = (int)all.size();
        r.pair = pair;
        for (int i = 0; i < n; i++) {
            const DevRep *d = reps[i];
            for (const Range *q : pick(d)) {
                if (q == nullptr || q->count <= 0) continue;
                for (int t = 0; t < q->count; t++) {
                    Tile m = d->tiles_host[q->first + t];
                    m.a = (uint64_t)i;
                    m.ld2 += map_off[i];
                    all.push_back(m);
                }
            }
        }
        r.count = (int)all.size() - r.first;
        if (r.count > 0) p->phases.push_back(r);
    };
    for (int s = 0; s < 3; s++) {
        merge(true, [&](const DevRep *d) { return std::vector<const Range *>{&d->den[s]}; });
        merge(false, [&](const DevRep *d) {
            std::vector<const Range *> v;
            for (int ln = 1; ln < kNfLanes; ln++) v.push_back(&d->den[ln * 3 + s]);
            return v;
        });
    }
    p->nf_phases = (int)p->phases.size();
    size_t nf = 0, nb = 0;
    for (int i = 0; i < n; i++) {
        nf = std::max(nf, reps[i]->fwd.size());
        nb = std::max(nb, reps[i]->bwd.size());
    }
    for (size_t k = 0; k < nf; k++)
        merge(true, [&](const DevRep *d) { return std::vector<const Range *>{k < d->fwd.size() ? &d->fwd[k] : nullptr}; });
    for (int s = 0; s < 3; s++)
        merge(false, [&](const DevRep *d) { return std::vector<const Range *>{&d->mid[s]}; });
    for (size_t k = 0; k < nb; k++)
        merge(true, [&](const DevRep *d) { return std::vector<const Range *>{k < d->bwd.size() ? &d->bwd[k] : nullptr}; });
    p->n_tiles = (int)all.size();
    const size_t map_bytes = 128;   /* sizeof(CUtensorMap) */
    if (cudaMalloc(&p->stiles, std::max<size_t>(all.size(), 1) * sizeof(Tile)) != cudaSuccess ||
        cudaMalloc(&p->maps, std::max<size_t>(n_maps, 1) * map_bytes) != cudaSuccess) {
        set_error("batch plan: device memory");
        return 10;
    }
    if (!all.empty() && cudaMemcpy(p->stiles, all.data(), all.size() * sizeof(Tile), cudaMemcpyHostToDevice) != cudaSuccess) {
        set_error("batch plan: tile upload");
        return 10;
    }
    for (int i = 0; i < n; i++) {
        const size_t cnt = std::max<size_t>(reps[i]->mixed_items.size(), 1);
        if (cudaMemcpy(static_cast<char *>(p->maps) + (size_t)map_off[i] * map_bytes, reps[i]->tmaps, cnt * map_bytes,
                       cudaMemcpyDeviceToDevice) != cudaSuccess) {
            set_error("batch plan: tensor map copy");
            return 10;
        }
    }
    return 0;
}

int build_plan(bool simt, int n, DevRep *const *reps, const int *n_den, BatchPlan **out)
{
    BatchPlan *p = new BatchPlan();
    p->simt = simt;
    std::vector<TileM> all;
    std::vector<std::pair<const int8_t *, int>> sc_src;   /* per merged range piece: source scales, count */
    std::vector<BatchMol> mols(n);
    for (int i = 0; i < n; i++) {
        p->reps.push_back(reps[i]);
        p->n_den.push_back(n_den[i]);
        p->bufs.push_back(reps[i]->xbuf);
        p->bufs.push_back(reps[i]->ybuf);
        p->bufs.push_back(reps[i]->work);
        p->plans.push_back(reps[i]->tiles);
        mols[i].va = rep_vecargs(reps[i], n_den[i]);
        mols[i].nvec = n_den[i];
        mols[i].pad_ = 0;
    }
    auto fail = [&](int rc) { delete p; return rc; };
    if (cudaMalloc(&p->mols, (size_t)std::max(n, 1) * sizeof(BatchMol)) != cudaSuccess ||
        cudaMemcpy(p->mols, mols.data(), (size_t)n * sizeof(BatchMol), cudaMemcpyHostToDevice) != cudaSuccess) {
        set_error("batch plan: structure table upload");
        return fail(10);
    }
    if (simt) {
        int rc = build_plan_simt(n, reps, n_den, p);
        if (rc) return fail(rc);
        *out = p;
        return 0;
    }
    /* one merged phase: the given range of every structure, in order */
    auto merge = [&](auto pick) {
        Range r;
        r.first = (int)all.size();
        for (int i = 0; i < n; i++) {
            const DevRep *d = reps[i];
            std::vector<const Range *> rs = pick(d);
            for (const Range *q : rs) {
                if (q == nullptr || q->count <= 0) continue;
                for (int t = 0; t < q->count; t++) {
                    TileM m = d->mtiles_host[q->first + t];
                    m.s_off = (uint64_t)(uintptr_t)d->mslices + m.s_off;
                    m.mol = i;
                    all.push_back(m);
                }
                sc_src.push_back({d->mscales + (size_t)q->first * 256, q->count});
            }
        }
        r.count = (int)all.size() - r.first;
        if (r.count > 0) p->phases.push_back(r);
    };
    for (int s = 0; s < 3; s++)
        merge([&](const DevRep *d) {
            std::vector<const Range *> v;
            for (int ln = 0; ln < kNfLanes; ln++) v.push_back(&d->mden[ln * 3 + s]);
            return v;
        });
    p->nf_phases = (int)p->phases.size();
    size_t nf = 0, nb = 0;
    for (int i = 0; i < n; i++) {
        nf = std::max(nf, reps[i]->mfwd.size());
        nb = std::max(nb, reps[i]->mbwd.size());
    }
    for (size_t k = 0; k < nf; k++)
        merge([&](const DevRep *d) {
            return std::vector<const Range *>{k < d->mfwd.size() ? &d->mfwd[k] : nullptr};
        });
    for (int s = 0; s < 3; s++)
        merge([&](const DevRep *d) { return std::vector<const Range *>{&d->mmid[s]}; });
    for (size_t k = 0; k < nb; k++)
        merge([&](const DevRep *d) {
            return std::vector<const Range *>{k < d->mbwd.size() ? &d->mbwd[k] : nullptr};
        });
    p->n_tiles = (int)all.size();
    if (cudaMalloc(&p->tiles, std::max<size_t>(all.size(), 1) * sizeof(TileM)) != cudaSuccess ||
        cudaMalloc(&p->scales, std::max<size_t>(all.size(), 1) * 256) != cudaSuccess) {
        set_error("batch plan: device memory");
        return fail(10);
    }
    if (!all.empty() &&
        cudaMemcpy(p->tiles, all.data(), all.size() * sizeof(TileM), cudaMemcpyHostToDevice) != cudaSuccess) {
        set_error("batch plan: tile upload");
        return fail(10);
    }
    size_t pos = 0;
    for (const auto &sp : sc_src) {
        if (cudaMemcpy(p->scales + pos * 256, sp.first, (size_t)sp.second * 256, cudaMemcpyDeviceToDevice) !=
            cudaSuccess) {
            set_error("batch plan: scale copy");
            return fail(10);
        }
        pos += (size_t)sp.second;
    }
    *out = p;
    return 0;
}

}  // namespace

/* 1: every structure runs the tensor-core kernel at its density count (its
 * own choice, default or tuned); 2 (only with H2G_BATCH_MERGED=1): every
 * structure runs the mixed single-density kernels and all have the same
 * density count; 0: otherwise (each structure then runs on its own
 * streams). */
int batch_merged_kind(int n, DevRep *const *reps, const int *n_den)
{
    if (n < 1) return 0;
    const char *e = std::getenv("H2G_BATCH_MERGED");
    if (e != nullptr && std::strcmp(e, "0") == 0) return 0;
    const bool force = e != nullptr && std::strcmp(e, "1") == 0;
    bool mma = true, simt = true;
    for (int i = 0; i < n; i++) {
        const DevRep *d = reps[i];
        if (d->precision != H2ERI_GPU_MIXED || d->device != reps[0]->device || d->tmaps == nullptr) return 0;
        if (d->mslices == nullptr || n_den[i] < d->cfg.mma_min_vec || n_den[i] > 16) mma = false;
        if (n_den[i] >= d->cfg.mma_min_vec && d->mslices != nullptr) simt = false;
        if (n_den[i] != n_den[0]) simt = false;
    }
    /* the single-density kernels' shared launches (kind 2) ran 7 % slower
     * than every structure on its own streams (64 alkanes C9..C59, two
     * densities each: 70.7 against 65.2 ms), so they run only on request */
    return mma ? 1 : (simt && force ? 2 : 0);
}

void batch_forget(const DevRep *d)
{
    std::lock_guard<std::mutex> lk(g_bmu);
    if (g_bplan == nullptr) return;
    for (const DevRep *r : g_bplan->reps)
        if (r == d) {
            delete g_bplan;
            g_bplan = nullptr;
            return;
        }
}

/* The batch on `s`: densities uncontracted per structure, the H2 products of
 * all structures phase by phase in shared launches, J contracted per
 * structure. Kernel errors (an expired bounded wait) are recorded in the
 * first structure's error word (H2ERI_gpu_check). */
int batch_coulomb_merged(int kind, int n, DevRep *const *reps, const int *n_den, const double *const *d_dens,
                         double *const *d_Js, cudaStream_t s)
{
    std::lock_guard<std::mutex> lk(g_bmu);
    const bool simt = kind == 2;
    for (int i = 0; i < n; i++) {
        int rc = ensure_work(reps[i], n_den[i]);
        if (rc) return rc;
    }
    if (!same_plan(g_bplan, simt, n, reps, n_den)) {
        delete g_bplan;
        g_bplan = nullptr;
        int rc = build_plan(simt, n, reps, n_den, &g_bplan);
        if (rc) return rc;
    }
    const BatchPlan *p = g_bplan;
    for (int i = 0; i < n; i++) {
        DevRep *d = reps[i];
        const size_t per = (size_t)2 * d->rank_total + d->lr_total;
        BCUDA_TRY(cudaMemsetAsync(d->work, 0, per * n_den[i] * sizeof(double), s));
        BCUDA_TRY(cudaMemsetAsync(d->ybuf, 0, (size_t)d->krnl * n_den[i] * sizeof(double), s));
        int rc = enqueue_uncontract(d, n_den[i], d_dens[i], s);
        if (rc) return rc;
    }
    /* the near-field phases on the first structure's low-priority stream,
     * beside the tree phases on s (as in the single-structure path: the near
     * field depends only on x, and its tiles fill the SMs the short tree
     * levels leave idle) */
    BatchPlan *pm = g_bplan;
    if (pm->ev_fork == nullptr) {
        BCUDA_TRY(cudaEventCreateWithFlags(&pm->ev_fork, cudaEventDisableTiming));
        BCUDA_TRY(cudaEventCreateWithFlags(&pm->ev_join, cudaEventDisableTiming));
    }
    cudaStream_t aux = reps[0]->s_aux;
    BCUDA_TRY(cudaEventRecord(pm->ev_fork, s));
    BCUDA_TRY(cudaStreamWaitEvent(aux, pm->ev_fork, 0));
    for (size_t k = 0; k < p->phases.size(); k++) {
        const Range &r = p->phases[k];
        cudaStream_t ls = (int)k < p->nf_phases ? aux : s;
        if (simt)
            launch_batch_mx(p->stiles + r.first, r.count, r.pair, p->maps, p->mols, n_den[0],
                            reps[0]->cfg.tiles_per_cta, reps[0]->err_flag_dev, ls);
        else
            launch_batch_mma(p->tiles + r.first, p->scales + (size_t)r.first * 256, p->mols, r.count,
                             reps[0]->mma_levels, reps[0]->n_sm, reps[0]->err_flag_dev, ls);
    }
    BCUDA_TRY(cudaGetLastError());
    BCUDA_TRY(cudaEventRecord(pm->ev_join, aux));
    BCUDA_TRY(cudaStreamWaitEvent(s, pm->ev_join, 0));
    for (int i = 0; i < n; i++) {
        int rc = enqueue_contract(reps[i], n_den[i], d_Js[i], s);
        if (rc) return rc;
    }
    return 0;
}

}  // namespace h2g
