/*
 * Autotuner of the H2 apply's launch choices.
 *
 * For one structure and one number of densities per launch, every candidate
 * launch configuration is run on the device and timed with CUDA events
 * (H2 matvecs on a fixed non-zero input, after warm-up), and the fastest is
 * kept in the structure's TuneCfg:
 *   single-density path (k_tile / k_tile_mx / k_tile_px): rows per tile
 *     (per range, or 512, 256, 128 for all: the tile plan is rebuilt from the
 *     recorded products);
 *     in the mixed mode one persistent launch, or a launch per range with
 *     tiles per CTA 2 or 1 and near-field lanes on their own streams or on
 *     one;
 *   several densities in the mixed mode: the tensor-core kernel (CTAs per
 *     launch n_SM or n_SM / 2, near-field lanes concurrent or not) against
 *     the single-density kernels, which decides the density count from
 *     which the tensor-core kernel runs.
 * Choices are cached per structure shape (basis functions, vector length,
 * nodes, blocks, sum of ranks), precision and density-count class, in the
 * process and, with H2G_TUNE_FILE=<path>, in a text file that later
 * processes read when a structure of the same shape is uploaded.
 */
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <mutex>
#include <sstream>
#include <string>
#include <vector>

#include "h2eri_gb300.h"
#include "h2g_gpu_api.h"

namespace h2g {

namespace {

std::mutex g_tmu;
std::map<std::string, TuneCfg> g_tcache;
bool g_tloaded = false;

int den_class(int n_den)
{
    if (n_den <= 1) return 1;
    if (n_den <= 3) return 2;
    if (n_den <= 7) return 4;
    if (n_den <= 15) return 8;
    return 16;
}

std::string tune_key(const DevRep *d, int n_den)
{
    std::ostringstream k;
    k << "bf" << d->num_bf << "_x" << d->krnl << "_n" << d->n_node << "_b" << d->n_B << "_d" << d->n_D << "_r"
      << d->rank_total << "_p" << d->precision << "_v" << den_class(n_den);
    return k.str();
}

void load_file_locked()
{
    if (g_tloaded) return;
    g_tloaded = true;
    const char *path = std::getenv("H2G_TUNE_FILE");
    if (path == nullptr || path[0] == '\0') return;
    std::ifstream f(path);
    std::string line;
    while (std::getline(f, line)) {
        /* key and five or six choices (files written before the persistent
         * kernel have five: it is then off) */
        std::istringstream ls(line);
        std::string key;
        TuneCfg c;
        if (!(ls >> key >> c.chunk_rows >> c.tiles_per_cta >> c.nf_concurrent >> c.mma_min_vec >> c.mma_grid_div))
            continue;
        if (!(ls >> c.persist)) c.persist = 0;
        g_tcache[key] = c;
    }
}

void save_locked(const std::string &key, const TuneCfg &c)
{
    g_tcache[key] = c;
    const char *path = std::getenv("H2G_TUNE_FILE");
    if (path == nullptr || path[0] == '\0') return;
    std::ofstream f(path, std::ios::app);
    f << key << ' ' << c.chunk_rows << ' ' << c.tiles_per_cta << ' ' << c.nf_concurrent << ' ' << c.mma_min_vec << ' '
      << c.mma_grid_div << ' ' << c.persist << '\n';
}

int apply_cfg(DevRep *d, const TuneCfg &c)
{
    int rc = replan_tiles(d, c.chunk_rows);
    if (rc) return rc;
    d->cfg = c;
    return 0;
}

/* ms per matvec of nvec vectors with the structure's current choices */
int time_matvec(DevRep *d, int nvec, double *ms)
{
    cudaStream_t s = d->s_main;
    cudaEvent_t e0, e1;
    if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
        set_error("autotune: cudaEventCreate failed");
        return 10;
    }
    int rc = 0;
    for (int i = 0; i < 2 && rc == 0; i++) rc = enqueue_matvec(d, nvec, d->xbuf, d->ybuf, s, false);
    if (rc == 0 && cudaStreamSynchronize(s) != cudaSuccess) rc = 10;
    int reps = 3;
    float t = 0.f;
    /* at least ~4 ms of device time per candidate */
    for (int round = 0; round < 4 && rc == 0; round++) {
        cudaEventRecord(e0, s);
        for (int i = 0; i < reps && rc == 0; i++) rc = enqueue_matvec(d, nvec, d->xbuf, d->ybuf, s, false);
        cudaEventRecord(e1, s);
        if (rc == 0 && cudaEventSynchronize(e1) != cudaSuccess) rc = 10;
        if (rc == 0) cudaEventElapsedTime(&t, e0, e1);
        if (t >= 4.0f) break;
        reps *= 4;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc == 0 && *d->err_flag != 0) {
        set_error("autotune: a tile kernel reported an expired wait");
        rc = 11;
    }
    if (rc) return rc;
    *ms = (double)t / reps;
    return 0;
}

}  // namespace

void tune_apply_cached(DevRep *d)
{
    std::lock_guard<std::mutex> lk(g_tmu);
    load_file_locked();
    /* the single-density choices, then the tensor-core choices of the
     * largest density class tuned for this shape */
    TuneCfg c = d->cfg;
    bool any = false;
    auto it = g_tcache.find(tune_key(d, 1));
    if (it != g_tcache.end()) {
        c.chunk_rows = it->second.chunk_rows;
        c.tiles_per_cta = it->second.tiles_per_cta;
        c.nf_concurrent = it->second.nf_concurrent;
        c.persist = it->second.persist;
        any = true;
    }
    for (int cls : {2, 4, 8, 16}) {
        auto jt = g_tcache.find(tune_key(d, cls));
        if (jt == g_tcache.end()) continue;
        c.mma_min_vec = jt->second.mma_min_vec;
        c.mma_grid_div = jt->second.mma_grid_div;
        any = true;
    }
    if (any) (void)apply_cfg(d, c);
}

}  // namespace h2g

using namespace h2g;

/* Runs the autotuner for h2eri at n_den densities per launch in its current
 * precision and keeps the fastest launch choices for it. out (n values at
 * most): [0] ms per matvec with the choice kept, [1] ms with the choices
 * before tuning, [2] number of candidates timed, [3..8] the choice (tile
 * rows, tiles per CTA, near-field lanes concurrent, density count from which
 * the tensor-core kernel runs, CTA divisor of its launches, persistent
 * launch), [9..] ms of every candidate in the order tried. Returns the number of values written,
 * or < 0 on error. */
extern "C" int H2ERI_gpu_autotune(H2ERI_p h2eri, int n_den, double *out, int n)
{
    H2gRange nvtx_range("H2ERI_gpu_autotune");
    if (n_den < 1 || n_den > 1024) { set_error("autotune: n_den out of range"); return -3; }
    DevRep *d;
    int rc = get_rep(h2eri, &d);
    if (rc) return -rc;
    rc = ensure_work(d, n_den);
    if (rc) return -rc;
    /* a fixed non-zero input (every byte 0x3F: about 4.8e-4) */
    if (cudaMemset(d->xbuf, 0x3F, (size_t)d->krnl * n_den * sizeof(double)) != cudaSuccess) {
        set_error("autotune: cudaMemset failed");
        return -10;
    }
    const TuneCfg start = d->cfg;
    std::vector<TuneCfg> cand;
    const bool mixed = d->precision == H2ERI_GPU_MIXED;
    /* the tensor-core kernel is a candidate where the current choices allow
     * it for this density count (its slices are made for the trial) */
    bool multi = mixed && n_den >= 2 && start.mma_min_vec <= n_den;
    if (multi) {
        rc = mma_make_slices(d);
        if (rc) return -rc;
        multi = d->mslices != nullptr;
    }
    cand.push_back(start);   /* the current choices first */
    if (multi) {
        for (int div : {1, 2})
            for (int nf : {1, 0}) {
                TuneCfg c = start;
                c.mma_min_vec = std::min(start.mma_min_vec, n_den);
                c.mma_grid_div = div;
                c.nf_concurrent = nf;
                cand.push_back(c);
            }
    }
    for (int rows : {0, 512, 256, 128}) {
        if (mixed) {
            /* one persistent launch (tiles per CTA and lanes do not apply) */
            TuneCfg c = start;
            c.chunk_rows = rows;
            c.persist = 1;
            if (multi) c.mma_min_vec = n_den + 1;
            cand.push_back(c);
        }
        for (int tpc : (mixed ? std::vector<int>{2, 1} : std::vector<int>{2}))
            for (int nf : {1, 0}) {
                TuneCfg c = start;
                c.chunk_rows = rows;
                c.tiles_per_cta = tpc;
                c.nf_concurrent = nf;
                c.persist = 0;
                if (multi) c.mma_min_vec = n_den + 1;   /* the single-density kernels for this count */
                cand.push_back(c);
            }
    }
    std::vector<double> ms(cand.size(), 1e300);
    size_t best = 0;
    for (size_t i = 0; i < cand.size(); i++) {
        rc = apply_cfg(d, cand[i]);
        if (rc == 0) rc = time_matvec(d, n_den, &ms[i]);
        if (rc) {
            const TuneCfg &c = cand[i];
            const std::string why = std::string(H2ERI_gpu_last_error()) + " (autotune candidate " + std::to_string(i) +
                                    ": tile rows " + std::to_string(c.chunk_rows) + ", tiles per CTA " +
                                    std::to_string(c.tiles_per_cta) + ", lanes concurrent " +
                                    std::to_string(c.nf_concurrent) + ", tensor-core kernel from " +
                                    std::to_string(c.mma_min_vec) + " densities, CTA divisor " +
                                    std::to_string(c.mma_grid_div) + ", persistent " + std::to_string(c.persist) + ")";
            (void)apply_cfg(d, start);
            set_error(why);
            return -rc;
        }
        if (ms[i] < ms[best]) best = i;
    }
    TuneCfg keep = cand[best];
    rc = apply_cfg(d, keep);
    if (rc) return -rc;
    {
        std::lock_guard<std::mutex> lk(g_tmu);
        load_file_locked();
        save_locked(tune_key(d, n_den), keep);
    }
    std::vector<double> v = {ms[best], ms[0], (double)cand.size(), (double)keep.chunk_rows,
                             (double)keep.tiles_per_cta, (double)keep.nf_concurrent, (double)keep.mma_min_vec,
                             (double)keep.mma_grid_div, (double)keep.persist};
    v.insert(v.end(), ms.begin(), ms.end());
    const int m = std::min(n, (int)v.size());
    for (int i = 0; i < m; i++) out[i] = v[i];
    return m;
}
