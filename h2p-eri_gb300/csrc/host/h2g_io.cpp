/*
 * Statistics report (H2P-ERI src/H2ERI_typedef.c:148-300) and a binary
 * save/load of the H2 representation. The file holds named blobs
 * (name, element size, count, bytes) so that fields can be added later
 * without breaking older readers.
 */
#include <cstdint>
#include <exception>
#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <utility>
#include <vector>
#include <omp.h>

#include "h2g_host.h"
#include "h2eri_gb300.h"
#include "h2g_gpu_stats.h"

using namespace h2g;

extern "C" void H2ERI_print_statistic(H2ERI_p h)
{
    if (h == nullptr) return;
    if (h->n_node == 0) {
        std::printf("H2ERI has nothing to report yet.\n");
        return;
    }
    std::printf("================ H2ERI molecular system info ================\n");
    std::printf("  * Number of atoms / shells / basis functions : %d, %d, %d\n", h->natom, h->nshell, h->num_bf);
    std::printf("  * Number of symm-unique screened shell pairs : %d\n", h->num_sp);
    std::printf("==================== H2ERI H2 tree info ====================\n");
    std::printf("  * Number of points               : %d\n", h->n_point);
    std::printf("  * Kernel matrix size             : %d\n", h->krnl_mat_size);
    std::printf("  * Maximum points in a leaf node  : %d\n", h->max_leaf_points);
    std::printf("  * Maximum leaf node box size     : %e\n", h->max_leaf_size);
    std::printf("  * Number of levels (root at 0)   : %d\n", h->max_level + 1);
    std::printf("  * Number of nodes                : %d\n", h->n_node);
    std::printf("  * Number of nodes on each level  : ");
    for (int i = 0; i <= h->max_level; i++) std::printf(i < h->max_level ? "%d, " : "%d\n", h->level_n_node[i]);
    std::printf("  * Number of nodes on each height : ");
    for (int i = 0; i <= h->max_level; i++) std::printf(i < h->max_level ? "%d, " : "%d\n", h->height_n_node[i]);
    std::printf("  * Minimum admissible pair level  : %d\n", h->min_adm_level);
    std::printf("  * Number of reduced adm. pairs   : %d\n", h->n_r_adm_pair);
    std::printf("  * Number of reduced inadm. pairs : %d\n", h->n_r_inadm_pair);
    if (h->U == nullptr) {
        std::printf("H2ERI H2 matrix has not been constructed yet.\n");
        return;
    }
    const double MB = 8.0 / 1048576.0;
    const size_t *ms = h->mat_size;
    std::printf("==================== H2ERI storage info ====================\n");
    std::printf("  * Just-In-Time B & D build      : No\n");
    std::printf("  * H2 representation U, B, D     : %.2lf, %.2lf, %.2lf (MB) \n", ms[U_SIZE_IDX] * MB,
                ms[B_SIZE_IDX] * MB, ms[D_SIZE_IDX] * MB);
    int max_rank = 0;
    double sum_rank = 0.0, nz = 0.0;
    for (int i = 0; i < h->n_UJ; i++) {
        int r = h->U[i]->ncol;
        if (r > 0) { sum_rank += r; nz += 1.0; max_rank = std::max(max_rank, r); }
    }
    std::printf("  * Max / Avg compressed rank     : %d, %.0lf \n", max_rank, nz > 0 ? sum_rank / nz : 0.0);
    std::printf("==================== H2ERI timing info =====================\n");
    const double *t = h->timers;
    std::printf("  * H2 construction time (sec)   = %.3lf \n",
                t[PT_TIMER_IDX] + t[U_BUILD_TIMER_IDX] + t[B_BUILD_TIMER_IDX] + t[D_BUILD_TIMER_IDX]);
    std::printf("      |----> Point partition     = %.3lf \n", t[PT_TIMER_IDX]);
    std::printf("      |----> U construction      = %.3lf \n", t[U_BUILD_TIMER_IDX]);
    std::printf("      |----> B construction      = %.3lf \n", t[B_BUILD_TIMER_IDX]);
    std::printf("      |----> D construction      = %.3lf \n", t[D_BUILD_TIMER_IDX]);
    if (h->n_matvec == 0) {
        std::printf("H2ERI does not have matvec timings results yet.\n");
    } else {
        /* GPU phases: timers hold device time per phase (CUDA events), the
         * byte model is the reference's mat_size[] accounting */
        double n = (double)h->n_matvec;
        const char *names[4] = {"Forward transformation     ", "Intermediate multiplication",
                                "Backward transformation    ", "Dense multiplication       "};
        double tot_t = 0.0, tot_b = 0.0;
        for (int k = 0; k < 4; k++) { tot_t += t[MV_FWD_TIMER_IDX + k] / n; tot_b += ms[MV_FWD_SIZE_IDX + k] * 8.0; }
        std::printf("  * H2 matvec average time (sec) = %.6lf, %.2lf GB/s (GPU)\n", tot_t, tot_b / tot_t / 1e9);
        for (int k = 0; k < 4; k++) {
            double tk = t[MV_FWD_TIMER_IDX + k] / n;
            std::printf("      |----> %s = %.6lf, %.2lf GB/s\n", names[k], tk,
                        tk > 0 ? ms[MV_FWD_SIZE_IDX + k] * 8.0 / tk / 1e9 : 0.0);
        }
        std::printf("      |----> Vector operations           = %.6lf\n", t[MV_VOP_TIMER_IDX] / n);
    }
    h2g_gpu_print_statistic(h);
    std::printf("=============================================================\n");
}

/* ======================================================================== */
/* save / load                                                               */
/* ======================================================================== */

namespace {

const char kMagic[8] = {'H', '2', 'G', 'R', 'E', 'P', '0', '1'};

struct Writer {
    FILE *f;
    bool ok = true;
    void blob(const char *name, const void *data, uint32_t esize, uint64_t count)
    {
        char nm[32] = {0};
        std::strncpy(nm, name, 31);
        ok = ok && std::fwrite(nm, 1, 32, f) == 32;
        ok = ok && std::fwrite(&esize, 4, 1, f) == 1;
        ok = ok && std::fwrite(&count, 8, 1, f) == 1;
        if (count > 0) ok = ok && std::fwrite(data, esize, count, f) == count;
    }
    void ints(const char *n, const int *p, size_t c) { blob(n, p, 4, c); }
    void dbls(const char *n, const double *p, size_t c) { blob(n, p, 8, c); }
};

}  // namespace

extern "C" int H2ERI_save_representation(H2ERI_p h, const char *path)
{
    if (h == nullptr || h->U == nullptr || h->c_D_blks == nullptr) return 1;
    FILE *f = std::fopen(path, "wb");
    if (f == nullptr) return 2;
    std::fwrite(kMagic, 1, 8, f);
    Writer w{f};
    int scal[] = {h->natom, h->nshell, h->max_am, h->max_shell_nbf, h->num_bf, h->num_sp, h->num_sp_bfp,
                  h->krnl_mat_size, h->n_point, h->n_node, h->root_idx, h->n_leaf_node, h->max_child,
                  h->max_level, h->min_adm_level, h->n_r_inadm_pair, h->n_r_adm_pair, h->n_UJ, h->n_B, h->n_D,
                  h->max_leaf_points};
    w.ints("scalars", scal, sizeof(scal) / sizeof(int));
    double dsc[] = {h->scr_tol, h->ext_tol, h->QR_stop_tol, h->max_leaf_size};
    w.dbls("dscalars", dsc, 4);
    const int nn = h->n_node, nl = h->max_level + 1;
    w.ints("shell_bf_sidx", h->shell_bf_sidx, h->nshell + 1);
    w.ints("sp_nbfp", h->sp_nbfp, h->num_sp);
    w.ints("sp_bfp_sidx", h->sp_bfp_sidx, h->num_sp + 1);
    w.ints("sp_shell_idx", h->sp_shell_idx, 2 * (size_t)h->num_sp);
    w.ints("node_adm_pairs_sidx", h->node_adm_pairs_sidx, nn + 1);
    w.ints("node_adm_pairs", h->node_adm_pairs, h->node_adm_pairs_sidx[nn]);
    w.ints("node_inadm_pairs_sidx", h->node_inadm_pairs_sidx, nn + 1);
    w.ints("node_inadm_pairs", h->node_inadm_pairs, h->node_inadm_pairs_sidx[nn]);
    w.ints("plist_sidx", h->plist_sidx, h->nshell + 1);
    w.ints("plist", h->plist, h->plist_sidx[h->nshell]);
    w.ints("plist_idx", h->plist_idx, h->plist_sidx[h->nshell]);
    w.ints("parent", h->parent, nn);
    w.ints("children", h->children, (size_t)nn * h->max_child);
    w.ints("pt_cluster", h->pt_cluster, 2 * (size_t)nn);
    w.ints("mat_cluster", h->mat_cluster, 2 * (size_t)nn);
    w.ints("n_child", h->n_child, nn);
    w.ints("node_level", h->node_level, nn);
    w.ints("node_height", h->node_height, nn);
    w.ints("level_n_node", h->level_n_node, nl);
    w.ints("level_nodes", h->level_nodes, (size_t)nl * h->n_leaf_node);
    w.ints("height_n_node", h->height_n_node, nl);
    w.ints("height_nodes", h->height_nodes, (size_t)nl * h->n_leaf_node);
    w.ints("r_inadm_pairs", h->r_inadm_pairs, 2 * (size_t)h->n_r_inadm_pair);
    w.ints("r_adm_pairs", h->r_adm_pairs, 2 * (size_t)h->n_r_adm_pair);
    w.ints("node_n_r_adm", h->node_n_r_adm, nn);
    w.ints("B_p2i_rowptr", h->B_p2i_rowptr, nn + 1);
    w.ints("B_p2i_colidx", h->B_p2i_colidx, h->B_p2i_rowptr[nn]);
    w.ints("B_p2i_val", h->B_p2i_val, h->B_p2i_rowptr[nn]);
    w.ints("D_p2i_rowptr", h->D_p2i_rowptr, nn + 1);
    w.ints("D_p2i_colidx", h->D_p2i_colidx, h->D_p2i_rowptr[nn]);
    w.ints("D_p2i_val", h->D_p2i_val, h->D_p2i_rowptr[nn]);
    w.ints("B_nrow", h->B_nrow, h->n_B);
    w.ints("B_ncol", h->B_ncol, h->n_B);
    w.ints("D_nrow", h->D_nrow, h->n_D);
    w.ints("D_ncol", h->D_ncol, h->n_D);
    w.blob("mat_size", h->mat_size, 8, 11);
    w.dbls("timers", h->timers, 4);
    auto mats = [&](const char *name, H2E_dense_mat_p *m, int n) {
        std::vector<int> hdr((size_t)n * 4);
        size_t tot = 0;
        for (int i = 0; i < n; i++) {
            hdr[4 * i] = m[i]->nrow; hdr[4 * i + 1] = m[i]->ncol; hdr[4 * i + 2] = m[i]->ld;
            int cnt = (m[i]->ld < 0) ? (m[i]->nrow + m[i]->ncol) * (-m[i]->ld) : m[i]->nrow * m[i]->ncol;
            hdr[4 * i + 3] = cnt;
            tot += (size_t)cnt;
        }
        std::string hn = std::string(name) + "_hdr";
        w.ints(hn.c_str(), hdr.data(), hdr.size());
        std::vector<double> all(tot);
        size_t off = 0;
        for (int i = 0; i < n; i++) {
            if (hdr[4 * i + 3] > 0) std::memcpy(all.data() + off, m[i]->data, sizeof(double) * hdr[4 * i + 3]);
            off += hdr[4 * i + 3];
        }
        w.dbls(name, all.data(), tot);
    };
    mats("U", h->U, h->n_UJ);
    mats("B", h->c_B_blks, h->n_B);
    mats("D", h->c_D_blks, h->n_D);
    bool ok = w.ok;
    std::fclose(f);
    return ok ? 0 : 3;
}

namespace {

/* Every blob the loader indexes must exist with its element size and at
 * least the count that the scalars imply, and every block header must match
 * the block data; a damaged file is rejected before anything is built from
 * it. */
bool blobs_consistent(const std::map<std::string, std::vector<char>> &blobs,
                      const std::map<std::string, uint32_t> &esz)
{
    auto has = [&](const std::string &n, uint32_t es, long long cnt) {
        auto it = blobs.find(n);
        auto ie = esz.find(n);
        return cnt >= 0 && it != blobs.end() && ie != esz.end() && ie->second == es &&
               it->second.size() >= (size_t)es * (size_t)cnt;
    };
    auto ival = [&](const std::string &n, size_t i) { return ((const int *)blobs.at(n).data())[i]; };
    if (!has("scalars", 4, 21) || !has("dscalars", 8, 4)) return false;
    const int *sc = (const int *)blobs.at("scalars").data();
    const long long ns = sc[1], nsp = sc[5], nn = sc[9], root = sc[10], nleaf = sc[11], maxc = sc[12],
                    maxl = sc[13], ninadm = sc[15], nadm = sc[16], nU = sc[17], nB = sc[18], nD = sc[19];
    for (int i = 0; i < 21; i++)
        if (sc[i] < 0 && i != 14) return false;   /* min_adm_level may be -1 */
    if (ns < 1 || nsp < 1 || nn < 1 || root >= nn || nleaf < 1 || maxc < 1 || nU > nn) return false;
    const long long nl = maxl + 1;
    struct Need { const char *name; long long cnt; };
    const Need fixed[] = {{"shell_bf_sidx", ns + 1}, {"sp_nbfp", nsp}, {"sp_bfp_sidx", nsp + 1},
                          {"sp_shell_idx", 2 * nsp}, {"node_adm_pairs_sidx", nn + 1},
                          {"node_inadm_pairs_sidx", nn + 1}, {"plist_sidx", ns + 1}, {"parent", nn},
                          {"children", nn * maxc}, {"pt_cluster", 2 * nn}, {"mat_cluster", 2 * nn},
                          {"n_child", nn}, {"node_level", nn}, {"node_height", nn}, {"level_n_node", nl},
                          {"level_nodes", nl * nleaf}, {"height_n_node", nl}, {"height_nodes", nl * nleaf},
                          {"r_inadm_pairs", 2 * ninadm}, {"r_adm_pairs", 2 * nadm}, {"node_n_r_adm", nn},
                          {"B_p2i_rowptr", nn + 1}, {"D_p2i_rowptr", nn + 1}, {"B_nrow", nB}, {"B_ncol", nB},
                          {"D_nrow", nD}, {"D_ncol", nD}};
    for (const Need &q : fixed)
        if (!has(q.name, 4, q.cnt)) return false;
    const long long nadmp = ival("node_adm_pairs_sidx", nn), ninp = ival("node_inadm_pairs_sidx", nn),
                    npl = ival("plist_sidx", ns), nbp = ival("B_p2i_rowptr", nn), ndp = ival("D_p2i_rowptr", nn);
    if (!has("node_adm_pairs", 4, nadmp) || !has("node_inadm_pairs", 4, ninp) || !has("plist", 4, npl) ||
        !has("plist_idx", 4, npl) || !has("B_p2i_colidx", 4, nbp) || !has("B_p2i_val", 4, nbp) ||
        !has("D_p2i_colidx", 4, ndp) || !has("D_p2i_val", 4, ndp) || !has("mat_size", 8, 11) ||
        !has("timers", 8, 4))
        return false;
    const std::pair<const char *, long long> mats[] = {{"U", nU}, {"B", nB}, {"D", nD}};
    for (const auto &m : mats) {
        const std::string hn = std::string(m.first) + "_hdr";
        if (!has(hn, 4, 4 * m.second)) return false;
        long long tot = 0;
        for (long long i = 0; i < m.second; i++) {
            const long long nr = ival(hn, 4 * i), nc = ival(hn, 4 * i + 1), ld = ival(hn, 4 * i + 2),
                            cnt = ival(hn, 4 * i + 3);
            if (nr < 0 || nc < 0 || cnt < 0) return false;
            if (ld < 0 ? cnt != (nr + nc) * -ld : (cnt != nr * nc || (nc > 0 && ld < nc))) return false;
            tot += cnt;
        }
        if (!has(m.first, 8, tot)) return false;
    }
    return true;
}

}  // namespace

extern "C" int H2ERI_load_representation(const char *path, H2ERI_p *h2eri_)
{
    FILE *f = std::fopen(path, "rb");
    if (f == nullptr) return 2;
    std::fseek(f, 0, SEEK_END);
    const long fsize = std::ftell(f);
    std::fseek(f, 0, SEEK_SET);
    char magic[8];
    if (fsize < 8 || std::fread(magic, 1, 8, f) != 8 || std::memcmp(magic, kMagic, 8) != 0) { std::fclose(f); return 4; }
    std::map<std::string, std::vector<char>> blobs;
    std::map<std::string, uint32_t> esz;
    try {
        while (true) {
            char nm[32];
            uint32_t es;
            uint64_t cnt;
            if (std::fread(nm, 1, 32, f) != 32) break;
            if (std::fread(&es, 4, 1, f) != 1 || std::fread(&cnt, 8, 1, f) != 1) { std::fclose(f); return 5; }
            /* sizes bounded by what is left of the file: no allocation from garbage */
            const long here = std::ftell(f);
            if ((es != 1 && es != 4 && es != 8) || cnt > (uint64_t)(fsize - here) / es) { std::fclose(f); return 5; }
            std::vector<char> buf((size_t)es * cnt);
            if (cnt > 0 && std::fread(buf.data(), es, cnt, f) != cnt) { std::fclose(f); return 5; }
            nm[31] = 0;
            blobs[nm] = std::move(buf);
            esz[nm] = es;
        }
    } catch (const std::exception &) {
        std::fclose(f);
        return 5;
    }
    std::fclose(f);
    if (!blobs_consistent(blobs, esz)) return 6;
    auto get_i = [&](const char *n) -> int * {
        auto it = blobs.find(n);
        H2G_CHECK(it != blobs.end(), "representation file lacks %s\n", n);
        int *p = (int *)std::malloc(std::max<size_t>(it->second.size(), 4));
        std::memcpy(p, it->second.data(), it->second.size());
        return p;
    };
    H2ERI_p h;
    const int *sc = (const int *)blobs.at("scalars").data();
    const double *dsc = (const double *)blobs.at("dscalars").data();
    H2ERI_init(&h, dsc[0], dsc[1], dsc[2]);
    h->natom = sc[0]; h->nshell = sc[1]; h->max_am = sc[2]; h->max_shell_nbf = sc[3]; h->num_bf = sc[4];
    h->num_sp = sc[5]; h->num_sp_bfp = sc[6]; h->krnl_mat_size = sc[7]; h->n_point = sc[8]; h->n_node = sc[9];
    h->root_idx = sc[10]; h->n_leaf_node = sc[11]; h->max_child = sc[12]; h->max_level = sc[13];
    h->min_adm_level = sc[14]; h->n_r_inadm_pair = sc[15]; h->n_r_adm_pair = sc[16]; h->n_UJ = sc[17];
    h->n_B = sc[18]; h->n_D = sc[19]; h->max_leaf_points = sc[20];
    h->max_leaf_size = dsc[3];
    h->shell_bf_sidx = get_i("shell_bf_sidx");
    h->sp_nbfp = get_i("sp_nbfp");
    h->sp_bfp_sidx = get_i("sp_bfp_sidx");
    h->sp_shell_idx = get_i("sp_shell_idx");
    h->node_adm_pairs_sidx = get_i("node_adm_pairs_sidx");
    h->node_adm_pairs = get_i("node_adm_pairs");
    h->node_inadm_pairs_sidx = get_i("node_inadm_pairs_sidx");
    h->node_inadm_pairs = get_i("node_inadm_pairs");
    h->plist_sidx = get_i("plist_sidx");
    h->plist = get_i("plist");
    h->plist_idx = get_i("plist_idx");
    h->parent = get_i("parent");
    h->children = get_i("children");
    h->pt_cluster = get_i("pt_cluster");
    h->mat_cluster = get_i("mat_cluster");
    h->n_child = get_i("n_child");
    h->node_level = get_i("node_level");
    h->node_height = get_i("node_height");
    h->level_n_node = get_i("level_n_node");
    h->level_nodes = get_i("level_nodes");
    h->height_n_node = get_i("height_n_node");
    h->height_nodes = get_i("height_nodes");
    h->r_inadm_pairs = get_i("r_inadm_pairs");
    h->r_adm_pairs = get_i("r_adm_pairs");
    h->node_n_r_adm = get_i("node_n_r_adm");
    h->B_p2i_rowptr = get_i("B_p2i_rowptr");
    h->B_p2i_colidx = get_i("B_p2i_colidx");
    h->B_p2i_val = get_i("B_p2i_val");
    h->D_p2i_rowptr = get_i("D_p2i_rowptr");
    h->D_p2i_colidx = get_i("D_p2i_colidx");
    h->D_p2i_val = get_i("D_p2i_val");
    h->B_nrow = get_i("B_nrow");
    h->B_ncol = get_i("B_ncol");
    h->D_nrow = get_i("D_nrow");
    h->D_ncol = get_i("D_ncol");
    std::memcpy(h->mat_size, blobs.at("mat_size").data(), 8 * 11);
    std::memcpy(h->timers, blobs.at("timers").data(), 8 * 4);
    h->index_seq = (int *)std::malloc(sizeof(int) * std::max(h->num_sp, 1));
    for (int i = 0; i < h->num_sp; i++) h->index_seq[i] = i;
    auto mats = [&](const char *name, int n) -> H2E_dense_mat_p * {
        const int *hdr = (const int *)blobs.at(std::string(name) + "_hdr").data();
        const double *all = (const double *)blobs.at(name).data();
        H2E_dense_mat_p *m = (H2E_dense_mat_p *)std::calloc(std::max(n, 1), sizeof(H2E_dense_mat_p));
        size_t off = 0;
        for (int i = 0; i < n; i++) {
            int nr = hdr[4 * i], nc = hdr[4 * i + 1], ld = hdr[4 * i + 2], cnt = hdr[4 * i + 3];
            if (ld < 0) {
                m[i] = dmat_new(1, cnt);
                m[i]->nrow = nr; m[i]->ncol = nc; m[i]->ld = ld;
            } else {
                m[i] = dmat_new(nr, nc);
                m[i]->ld = ld;
            }
            if (cnt > 0) std::memcpy(m[i]->data, all + off, sizeof(double) * cnt);
            off += (size_t)cnt;
        }
        return m;
    };
    h->U = mats("U", h->n_UJ);
    h->c_B_blks = mats("B", h->n_B);
    h->c_D_blks = mats("D", h->n_D);
    /* work partitions and thread buffers, as H2ERI_build_H2 leaves them */
    std::vector<size_t> sz(std::max(h->n_D, std::max(h->n_B, 1)));
    size_t tot = 0;
    for (int i = 0; i < h->n_B; i++) { sz[i] = (size_t)h->c_B_blks[i]->size; tot += sz[i]; }
    partition_workload(h->n_B, sz.data(), tot, h->n_thread, h->B_blk);
    size_t t0 = 0, t1 = 0;
    for (int i = 0; i < h->n_D; i++) { sz[i] = (size_t)h->c_D_blks[i]->size; (i < h->n_leaf_node ? t0 : t1) += sz[i]; }
    partition_workload(h->n_leaf_node, sz.data(), t0, h->n_thread, h->D_blk0);
    partition_workload(h->n_r_inadm_pair, sz.data() + h->n_leaf_node, t1, h->n_thread, h->D_blk1);
    h->thread_buffs = (H2E_thread_buf_p *)std::malloc(sizeof(H2E_thread_buf_p) * h->n_thread);
    for (int i = 0; i < h->n_thread; i++) h->thread_buffs[i] = tbuf_new(h->krnl_mat_size);
    *h2eri_ = h;
    return 0;
}

extern "C" void H2ERI_exchange_workbuf_init(H2ERI_p h2eri) { (void)h2eri; }
extern "C" void H2ERI_exchange_workbuf_free(H2ERI_p h2eri)
{
    /* The GPU exchange never allocates a host work buffer. */
    (void)h2eri;
}
