/*
 * Per-geometry set-up on the host: structure life cycle, .mol input, shell-pair
 * screening and extents, hierarchical partitioning. These run once per
 * geometry before the H2 blocks are uploaded to the GPU; they restate the
 * reference algorithms so that the same tree, pair lists and vector ordering
 * come out (references per function below).
 */
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <sys/time.h>
#include <omp.h>

#include "h2g_host.h"
#include "h2eri_gb300.h"

namespace h2g {

double wtime()
{
    struct timeval tv;
    gettimeofday(&tv, nullptr);
    return tv.tv_sec + 1e-6 * tv.tv_usec;
}

void *amalloc(size_t bytes)
{
    void *p = nullptr;
    if (posix_memalign(&p, 64, bytes > 0 ? bytes : 64) != 0) p = nullptr;
    H2G_CHECK(p != nullptr, "allocation of %zu bytes failed\n", bytes);
    return p;
}

H2E_int_vec_p ivec_new(int capacity)
{
    if (capacity < 0) capacity = 128;
    H2E_int_vec_p v = (H2E_int_vec_p)std::malloc(sizeof(struct H2E_int_vec));
    H2G_CHECK(v != nullptr, "ivec alloc\n");
    v->data = (int *)std::malloc(sizeof(int) * (size_t)(capacity > 0 ? capacity : 1));
    H2G_CHECK(v->data != nullptr, "ivec data alloc\n");
    v->capacity = capacity;
    v->length = 0;
    return v;
}

void ivec_free(H2E_int_vec_p *v)
{
    if (*v == nullptr) return;
    std::free((*v)->data);
    std::free(*v);
    *v = nullptr;
}

void ivec_reserve(H2E_int_vec_p v, int capacity)
{
    if (capacity <= v->capacity) return;
    int *d = (int *)std::malloc(sizeof(int) * (size_t)capacity);
    H2G_CHECK(d != nullptr, "ivec grow to %d\n", capacity);
    if (v->length > 0) std::memcpy(d, v->data, sizeof(int) * (size_t)v->length);
    std::free(v->data);
    v->data = d;
    v->capacity = capacity;
}

void ivec_push(H2E_int_vec_p v, int x)
{
    if (v->length == v->capacity) ivec_reserve(v, v->capacity > 0 ? 2 * v->capacity : 16);
    v->data[v->length++] = x;
}

H2E_dense_mat_p dmat_new(int nrow, int ncol)
{
    H2E_dense_mat_p m = (H2E_dense_mat_p)std::malloc(sizeof(struct H2E_dense_mat));
    H2G_CHECK(m != nullptr, "dmat alloc\n");
    m->nrow = std::max(0, nrow);
    m->ncol = std::max(0, ncol);
    m->ld = m->ncol;
    m->size = m->nrow * m->ncol;
    m->data = (m->size > 0) ? (double *)amalloc(sizeof(double) * (size_t)m->size) : nullptr;
    return m;
}

void dmat_free(H2E_dense_mat_p *m)
{
    if (*m == nullptr) return;
    std::free((*m)->data);
    std::free(*m);
    *m = nullptr;
}

void dmat_resize(H2E_dense_mat_p m, int nrow, int ncol)
{
    int sz = nrow * ncol;
    m->nrow = nrow;
    m->ncol = ncol;
    m->ld = ncol;
    if (sz > m->size) {
        std::free(m->data);
        m->data = (double *)amalloc(sizeof(double) * (size_t)sz);
        m->size = sz;
    }
}

H2E_thread_buf_p tbuf_new(int krnl_mat_size)
{
    H2E_thread_buf_p tb = (H2E_thread_buf_p)std::malloc(sizeof(struct H2E_thread_buf));
    H2G_CHECK(tb != nullptr, "thread buffer alloc\n");
    tb->idx0 = ivec_new(1024);
    tb->idx1 = ivec_new(1024);
    tb->mat0 = dmat_new(1024, 1);
    tb->mat1 = dmat_new(1024, 1);
    tb->mat2 = dmat_new(1024, 1);
    tb->y = (double *)amalloc(sizeof(double) * (size_t)std::max(krnl_mat_size, 1));
    tb->timer = 0.0;
    return tb;
}

void tbuf_free(H2E_thread_buf_p *tb)
{
    if (*tb == nullptr) return;
    ivec_free(&(*tb)->idx0);
    ivec_free(&(*tb)->idx1);
    dmat_free(&(*tb)->mat0);
    dmat_free(&(*tb)->mat1);
    dmat_free(&(*tb)->mat2);
    std::free((*tb)->y);
    std::free(*tb);
    *tb = nullptr;
}

void tbuf_reset(H2E_thread_buf_p tb)
{
    if (tb == nullptr) return;
    H2E_int_vec_p *iv[2] = {&tb->idx0, &tb->idx1};
    for (auto p : iv) { ivec_free(p); *p = ivec_new(128); }
    H2E_dense_mat_p *dm[3] = {&tb->mat0, &tb->mat1, &tb->mat2};
    for (auto p : dm) { dmat_free(p); *p = dmat_new(0, 0); }
}

void partition_workload(int n_work, const size_t *work_sizes, size_t total, int n_block,
                        H2E_int_vec_p displs)
{
    ivec_reserve(displs, n_block + 1);
    displs->data[0] = 0;
    for (int i = 1; i < displs->capacity; i++) displs->data[i] = n_work;
    size_t blk = total / (size_t)n_block + 1, cur = 0;
    int idx = 1;
    for (int i = 0; i < n_work; i++) {
        cur += work_sizes[i];
        if (cur >= blk) {
            displs->data[idx++] = i + 1;
            cur = 0;
        }
    }
    if (cur > 0) displs->data[idx++] = n_work;
    displs->length = idx;
}

/* ---------------------------------------------------------------------- */
/* Integral helpers                                                        */
/* ---------------------------------------------------------------------- */

h2g_pair *sp_pair(H2ERI_p h2eri, int sp_idx)
{
    return (h2g_pair *)h2eri->sp[sp_idx].pairs[0];
}

/* Matrix of shell quartets (N_i M_i | Q_j P_j) unfolded row by row
 * (H2P-ERI src/CMS.c:387-451). */
void eri_pairs_to_mat(H2ERI_p h2eri, int n_bra, const int *bra, int n_ket, const int *ket,
                      double *mat, int ldm)
{
    double buf[15 * 15 * 15 * 15];
    int row = 0;
    for (int i = 0; i < n_bra; i++) {
        const h2g_pair *bp = sp_pair(h2eri, bra[i]);
        int nr = h2g_ncart(bp->am1) * h2g_ncart(bp->am2);
        int col = 0;
        for (int j = 0; j < n_ket; j++) {
            const h2g_pair *kp = sp_pair(h2eri, ket[j]);
            int nc = h2g_ncart(kp->am1) * h2g_ncart(kp->am2);
            h2g_eri_quartet(bp, kp, buf);
            for (int r = 0; r < nr; r++)
                std::memcpy(mat + (size_t)(row + r) * ldm + col, buf + (size_t)r * nc, sizeof(double) * nc);
            col += nc;
        }
        row += nr;
    }
}

/* Potential integrals (N_i M_i | point_j) as an (SSP bf pairs) x n_pt matrix
 * (H2P-ERI src/CMS.c:455-482). */
void nai_pairs_to_mat(H2ERI_p h2eri, int n_bra, const int *bra, int n_pt,
                      const double *x, const double *y, const double *z, double *mat, int ldm)
{
    int num_sp = h2eri->num_sp;
    int row = 0;
    for (int i = 0; i < n_bra; i++) {
        const shell_t *Ms = h2eri->sp_shells + bra[i];
        const shell_t *Ns = h2eri->sp_shells + bra[i] + num_sp;
        h2g_shell M = {Ms->am, Ms->nprim, Ms->x, Ms->y, Ms->z, Ms->alpha, Ms->coef};
        h2g_shell N = {Ns->am, Ns->nprim, Ns->x, Ns->y, Ns->z, Ns->alpha, Ns->coef};
        h2g_potential_points(&N, &M, n_pt, x, y, z, 1.0, mat + (size_t)row * ldm, ldm);
        row += h2g_ncart(M.am) * h2g_ncart(N.am);
    }
}

}  // namespace h2g

using namespace h2g;

/* ======================================================================== */
/* Life cycle                                                                */
/* ======================================================================== */

static int env_int(const char *name, int def, int lo, int hi)
{
    const char *s = std::getenv(name);
    if (s == nullptr) return def;
    int v = std::atoi(s);
    return (v < lo || v > hi) ? def : v;
}

extern "C" void H2ERI_init(H2ERI_p *h2eri_, const double scr_tol, const double ext_tol, const double QR_tol)
{
    h2g_ints_init();
    H2ERI_p h = (H2ERI_p)std::calloc(1, sizeof(struct H2ERI));
    H2G_CHECK(h != nullptr, "H2ERI alloc\n");
    h->scr_tol = scr_tol;
    h->ext_tol = ext_tol;
    h->pp_npts_layer = 384;
    h->pp_nlayer_ext = 3;
    h->n_thread = omp_get_max_threads();
    h->pt_dim = 3;
    h->xpt_dim = 3;
    h->krnl_dim = 1;
    h->max_child = 8;
    h->max_neighbor = 27;
    h->QR_stop_type = 1;           /* relative column norm */
    h->QR_stop_tol = QR_tol;
    h->B_blk = ivec_new(h->n_thread * H2G_BD_NTASK + 5);
    h->D_blk0 = ivec_new(h->n_thread * H2G_BD_NTASK + 5);
    h->D_blk1 = ivec_new(h->n_thread * H2G_BD_NTASK + 5);
    h->print_timers = env_int("H2E_PRINT_TIMERS", 0, 0, 1);
    h->print_dbginfo = env_int("H2E_PRINT_DBGINFO", 0, 0, 1);
    *h2eri_ = h;
}

static void free_shells(int n, shell_t *s)
{
    if (s == nullptr) return;
    for (int i = 0; i < n; i++) {
        std::free(s[i].alpha);
        std::free(s[i].coef);
    }
}

extern "C" void H2ERI_destroy(H2ERI_p h)
{
    if (h == nullptr) return;
    H2ERI_gpu_release(h);
    int *int_arrays[] = {
        h->shell_bf_sidx, h->sp_nbfp, h->sp_bfp_sidx, h->sp_shell_idx, h->index_seq,
        h->node_adm_pairs, h->node_adm_pairs_sidx, h->node_inadm_pairs, h->node_inadm_pairs_sidx,
        h->plist, h->plist_idx, h->plist_sidx, h->dlist, h->dlist_sidx,
        h->parent, h->children, h->pt_cluster, h->mat_cluster, h->n_child, h->node_level,
        h->node_height, h->level_n_node, h->level_nodes, h->height_n_node, h->height_nodes,
        h->r_inadm_pairs, h->r_adm_pairs, h->node_inadm_lists, h->node_n_r_inadm, h->node_n_r_adm,
        h->coord_idx, h->B_p2i_rowptr, h->B_p2i_colidx, h->B_p2i_val, h->D_p2i_rowptr,
        h->D_p2i_colidx, h->D_p2i_val, h->B_nrow, h->B_ncol, h->D_nrow, h->D_ncol};
    for (int *p : int_arrays) std::free(p);
    double *dbl_arrays[] = {h->sp_center, h->sp_extent, h->box_extent, h->unc_denmat_x, h->H2_matvec_y,
                            h->coord, h->coord0, h->enbox, h->root_enbox, h->B_data, h->D_data};
    for (double *p : dbl_arrays) std::free(p);
    std::free(h->B_ptr);
    std::free(h->D_ptr);
    free_shells(h->nshell, h->shells);
    free_shells(h->num_sp * 2, h->sp_shells);
    std::free(h->shells);
    std::free(h->sp_shells);
    if (h->sp != nullptr) {
        for (int i = 0; i < h->num_sp; i++) {
            for (int k = 0; k < h->sp[i].nshell12; k++) {
                h2g_pair_free((h2g_pair *)h->sp[i].pairs[k]);
                std::free(h->sp[i].pairs[k]);
            }
            std::free(h->sp[i].pairs);
        }
        std::free(h->sp);
    }
    auto free_ivecs = [&](H2E_int_vec_p *arr) {
        if (arr == nullptr) return;
        for (int i = 0; i < h->n_node; i++) ivec_free(&arr[i]);
        std::free(arr);
    };
    free_ivecs(h->J_pair);
    free_ivecs(h->J_row);
    free_ivecs(h->ovlp_ff_idx);
    if (h->thread_buffs != nullptr) {
        for (int i = 0; i < h->n_thread; i++) tbuf_free(&h->thread_buffs[i]);
        std::free(h->thread_buffs);
    }
    auto free_dmats = [](H2E_dense_mat_p *arr, int n) {
        if (arr == nullptr) return;
        for (int i = 0; i < n; i++) dmat_free(&arr[i]);
        std::free(arr);
    };
    free_dmats(h->c_B_blks, h->n_B);
    free_dmats(h->c_D_blks, h->n_D);
    free_dmats(h->U, h->n_UJ);
    free_dmats(h->y0, h->n_node);
    free_dmats(h->y1, h->n_node);
    ivec_free(&h->B_blk);
    ivec_free(&h->D_blk0);
    ivec_free(&h->D_blk1);
    std::free(h);
}

extern "C" void H2E_reset_timers(H2ERI_p h)
{
    h->n_matvec = 0;
    h->mat_size[MV_VOP_SIZE_IDX] = 0;
    for (int i = MV_FWD_TIMER_IDX; i <= MV_VOP_TIMER_IDX; i++) h->timers[i] = 0.0;
}

/* ======================================================================== */
/* .mol input (H2P-ERI src/CMS.c:14-123)                                     */
/* ======================================================================== */

extern "C" void CMS_read_mol_file(const char *mol_fname, int *natom_, int *nshell_, shell_t **shells_)
{
    h2g_ints_init();
    FILE *f = std::fopen(mol_fname, "r");
    H2G_CHECK(f != nullptr, "cannot open mol file %s\n", mol_fname);
    auto am_of = [](char c) -> int {
        const char *tbl = "SPDFGHIJKL";
        const char *p = std::strchr(tbl, c);
        H2G_CHECK(p != nullptr && c != 0, "unknown shell type %c\n", c);
        return (int)(p - tbl);
    };
    int natom = 0;
    H2G_CHECK(std::fscanf(f, "%d", &natom) == 1 && natom >= 0, "bad mol header\n");
    std::vector<shell_t> shells;
    for (int a = 0; a < natom; a++) {
        char sym[16];
        int nshell, nprimall, nallprimg;
        double x, y, z;
        H2G_CHECK(std::fscanf(f, "%15s %d %d %d", sym, &nshell, &nprimall, &nallprimg) == 4 && nshell >= 0,
                  "bad atom header\n");
        H2G_CHECK(std::fscanf(f, "%lf %lf %lf", &x, &y, &z) == 3, "bad coordinates\n");
        for (int s = 0; s < nshell; s++) {
            char type[16];
            int nprim, ngen;
            H2G_CHECK(std::fscanf(f, "%15s %d %d", type, &nprim, &ngen) == 3 && nprim >= 1, "bad shell header\n");
            H2G_CHECK(ngen >= 1 && ngen <= (int)std::strlen(type), "bad contraction count\n");
            size_t base = shells.size();
            for (int g = 0; g < ngen; g++) {
                shell_t sh;
                std::memset(&sh, 0, sizeof(sh));
                sh.am = am_of(type[g]);
                H2G_CHECK(sh.am <= H2G_MAX_AM, "angular momentum %d above supported %d\n", sh.am, H2G_MAX_AM);
                sh.nprim = nprim;
                sh.x = x; sh.y = y; sh.z = z;
                sh.alpha = (double *)std::calloc((size_t)nprim, sizeof(double));
                sh.coef = (double *)std::calloc((size_t)nprim, sizeof(double));
                shells.push_back(sh);
            }
            for (int k = 0; k < nprim; k++) {
                double alpha;
                H2G_CHECK(std::fscanf(f, "%lf", &alpha) == 1, "bad exponent\n");
                for (int g = 0; g < ngen; g++) {
                    double c;
                    H2G_CHECK(std::fscanf(f, "%lf", &c) == 1, "bad coefficient\n");
                    shells[base + g].alpha[k] = alpha;
                    shells[base + g].coef[k] = c;
                }
            }
        }
    }
    std::fclose(f);
    for (auto &s : shells) h2g_normalize_shell(s.am, s.nprim, s.alpha, s.coef);
    shell_t *out = (shell_t *)std::malloc(sizeof(shell_t) * std::max<size_t>(shells.size(), 1));
    std::memcpy(out, shells.data(), sizeof(shell_t) * shells.size());
    *natom_ = natom;
    *nshell_ = (int)shells.size();
    *shells_ = out;
}

extern "C" void CMS_destroy_shells(const int nshell, shell_t *shells) { free_shells(nshell, shells); }

static void copy_shell(const shell_t *src, shell_t *dst)
{
    *dst = *src;
    dst->alpha = (double *)std::malloc(sizeof(double) * (size_t)src->nprim);
    dst->coef = (double *)std::malloc(sizeof(double) * (size_t)src->nprim);
    std::memcpy(dst->alpha, src->alpha, sizeof(double) * (size_t)src->nprim);
    std::memcpy(dst->coef, src->coef, sizeof(double) * (size_t)src->nprim);
}

static h2g_shell as_h2g(const shell_t *s)
{
    h2g_shell t = {s->am, s->nprim, s->x, s->y, s->z, s->alpha, s->coef};
    return t;
}

/* ======================================================================== */
/* Shell-pair screening and extents (H2P-ERI src/H2ERI_shell_operations.c)  */
/* ======================================================================== */

/* Schwarz values: for each shell pair the maximum of |(MN|MN)| over the
 * entries the reference inspects (src/CMS.c:163-229: pair (M,N), entries
 * iN*(dM*dN*dM+dM) + iM*(dN*dM+1)). For M > N the (M,N) evaluation is kept,
 * i.e. the later write of the reference's loop over all ordered pairs. */
static void schwarz_values(H2ERI_p h, std::vector<double> &scr, double &max_val)
{
    int n = h->nshell;
    scr.assign((size_t)n * n, 0.0);
    double gmax = 0.0;
    #pragma omp parallel for schedule(dynamic) reduction(max : gmax)
    for (int M = 0; M < n; M++) {
        std::vector<double> eri(15 * 15 * 15 * 15);
        for (int N = 0; N <= M; N++) {
            h2g_shell a = as_h2g(&h->shells[M]), b = as_h2g(&h->shells[N]);
            h2g_pair pr;
            h2g_pair_init(&pr, &a, &b);
            h2g_eri_quartet(&pr, &pr, eri.data());
            h2g_pair_free(&pr);
            int dM = NCART(a.am), dN = NCART(b.am);
            double v = 0.0;
            for (int iM = 0; iM < dM; iM++)
                for (int iN = 0; iN < dN; iN++) {
                    int idx = iN * (dM * dN * dM + dM) + iM * (dN * dM + 1);
                    v = std::max(v, std::fabs(eri[idx]));
                }
            scr[(size_t)M * n + N] = v;
            scr[(size_t)N * n + M] = v;
            gmax = std::max(gmax, v);
        }
    }
    max_val = gmax;
}

static void screen_shell_pairs(H2ERI_p h)
{
    int n = h->nshell;
    std::vector<double> scr;
    double max_val = 0.0;
    schwarz_values(h, scr, max_val);
    double thres = h->scr_tol * h->scr_tol / max_val;
    int num_sp = 0;
    for (int i = 0; i < n; i++)
        for (int j = i; j < n; j++)
            if (scr[(size_t)i * n + j] >= thres) num_sp++;
    h->num_sp = num_sp;
    h->sp_shells = (shell_t *)std::calloc((size_t)num_sp * 2, sizeof(shell_t));
    h->sp_shell_idx = (int *)std::malloc(sizeof(int) * (size_t)num_sp * 2);
    int k = 0;
    for (int i = 0; i < n; i++)
        for (int j = i; j < n; j++) {
            if (scr[(size_t)i * n + j] < thres) continue;
            copy_shell(&h->shells[i], &h->sp_shells[k]);
            copy_shell(&h->shells[j], &h->sp_shells[k + num_sp]);
            h->sp_shell_idx[k] = i;
            h->sp_shell_idx[k + num_sp] = j;
            k++;
        }
}

/* Radius r beyond which coef * exp(-alpha r^2) r^am < tol, by bisection
 * (src/H2ERI_shell_operations.c:99-128). */
static double gaussian_extent(double alpha, double coef, int am_i, double tol)
{
    const double am = (double)am_i;
    auto g = [&](double x) { return coef * std::exp(-alpha * x * x) * std::pow(x, am) - tol; };
    double lo = 0.0, hi = 20.0;
    if (am_i > 0) {
        lo = std::sqrt(am * 0.5 / alpha);
        hi = 10.0 * lo;
    }
    if (g(lo) <= 1e-8 * tol) return 0.0;
    while (g(hi) > 0) hi *= 2.0;
    double r = 0.5 * (lo + hi), gr = g(r);
    while (std::fabs(gr) > 2e-16) {
        if (gr > 0.0) lo = r; else hi = r;
        r = 0.5 * (lo + hi);
        gr = g(r);
    }
    return r;
}

/* Extent and centre of each SSP (src/H2ERI_shell_operations.c:137-310). */
static void calc_sp_extents(H2ERI_p h)
{
    int num_sp = h->num_sp;
    h->sp_extent = (double *)std::malloc(sizeof(double) * (size_t)num_sp);
    h->sp_center = (double *)std::malloc(sizeof(double) * (size_t)num_sp * 3);
    double *ext = h->sp_extent, *cen = h->sp_center;
    for (int i = 0; i < num_sp; i++) {
        const shell_t *s0 = h->sp_shells + i, *s1 = h->sp_shells + i + num_sp;
        int np0 = s0->nprim, np1 = s1->nprim, np01 = np0 * np1, am01 = s0->am + s1->am;
        double dx = s0->x - s1->x, dy = s0->y - s1->y, dz = s0->z - s1->z;
        double tol_i = h->ext_tol / (double)np01;
        double r01 = dx * dx + dy * dy + dz * dz, d01 = std::sqrt(r01);
        std::vector<double> e(np01), c(3 * (size_t)np01);
        double emax = 0.0;
        for (int j0 = 0; j0 < np0; j0++)
            for (int j1 = 0; j1 < np1; j1++) {
                double a0 = s0->alpha[j0], a1 = s1->alpha[j1], ap = a0 + a1;
                double coef = s0->coef[j0] * s1->coef[j1] * std::exp(-a0 * a1 / ap * r01);
                int j = j0 * np1 + j1;
                e[j] = gaussian_extent(ap, coef, am01, tol_i);
                emax = std::max(emax, e[j]);
                c[0 * np01 + j] = (a0 * s0->x + a1 * s1->x) / ap;
                c[1 * np01 + j] = (a0 * s0->y + a1 * s1->y) / ap;
                c[2 * np01 + j] = (a0 * s0->z + a1 * s1->z) / ap;
            }
        if (d01 < 1e-16) {
            ext[i] = emax;
            cen[i] = s0->x; cen[num_sp + i] = s0->y; cen[2 * num_sp + i] = s0->z;
            continue;
        }
        if (emax < 1e-16) {
            double sx = 0, sy = 0, sz = 0;
            for (int j = 0; j < np01; j++) { sx += c[j]; sy += c[np01 + j]; sz += c[2 * np01 + j]; }
            ext[i] = 0.0;
            cen[i] = sx / np01; cen[num_sp + i] = sy / np01; cen[2 * num_sp + i] = sz / np01;
            continue;
        }
        dx /= d01; dy /= d01; dz /= d01;
        /* primitive extents as segments along the A-B axis; keep the
         * upper end farthest from B and the lower end farthest from A */
        int j0 = -1, j1 = -1;
        double m0 = 0.0, m1 = 0.0;
        double up[3] = {0, 0, 0}, lo[3] = {0, 0, 0};
        for (int j = 0; j < np01; j++) {
            if (e[j] <= 1e-16) continue;
            double ux = c[j] + e[j] * dx, uy = c[np01 + j] + e[j] * dy, uz = c[2 * np01 + j] + e[j] * dz;
            double lx = c[j] - e[j] * dx, ly = c[np01 + j] - e[j] * dy, lz = c[2 * np01 + j] - e[j] * dz;
            double q0 = (ux - s1->x) * (ux - s1->x) + (uy - s1->y) * (uy - s1->y) + (uz - s1->z) * (uz - s1->z);
            if (q0 > m0) { m0 = q0; j0 = j; up[0] = ux; up[1] = uy; up[2] = uz; }
            double q1 = (lx - s0->x) * (lx - s0->x) + (ly - s0->y) * (ly - s0->y) + (lz - s0->z) * (lz - s0->z);
            if (q1 > m1) { m1 = q1; j1 = j; lo[0] = lx; lo[1] = ly; lo[2] = lz; }
        }
        (void)j0; (void)j1;
        double wx = up[0] - lo[0], wy = up[1] - lo[1], wz = up[2] - lo[2];
        ext[i] = 0.5 * std::sqrt(wx * wx + wy * wy + wz * wz);
        cen[i] = 0.5 * (up[0] + lo[0]);
        cen[num_sp + i] = 0.5 * (up[1] + lo[1]);
        cen[2 * num_sp + i] = 0.5 * (up[2] + lo[2]);
    }
}

extern "C" void H2ERI_process_shells(H2ERI_p h2eri)
{
    screen_shell_pairs(h2eri);
    calc_sp_extents(h2eri);
}

/* ======================================================================== */
/* Hierarchical partitioning (src/H2ERI_partition_points.c,                  */
/* src/H2ERI_partition.c)                                                    */
/* ======================================================================== */

namespace {

struct TreeNode {
    int n_child = 0, n_node = 1, po_idx = 0, level = 0, height = 0;
    int pt_s = 0, pt_e = -1;
    double enbox[6];
    TreeNode *child[8] = {nullptr};
    ~TreeNode() { for (auto c : child) delete c; }
};

struct PartVars {
    int curr_po_idx = 0, max_level = 0, n_leaf = 0;
};

/* Recursive 2^3-way bisection; nodes numbered in post order
 * (src/H2ERI_partition_points.c:36-265). */
TreeNode *bisect(int level, int cs, int ce, int n_point, double max_leaf_size, int max_leaf_points,
                 const double *enbox_in, double *coord, double *coord_tmp, int *cidx, int *cidx_tmp,
                 PartVars &pv)
{
    const int dim = 3;
    int npts = ce - cs + 1;
    pv.max_level = std::max(pv.max_level, level);
    double enbox[6];
    if (enbox_in == nullptr) {
        double center[3] = {0, 0, 0};
        for (int j = 0; j < dim; j++)
            for (int i = cs; i <= ce; i++) center[j] += coord[j * n_point + i];
        for (int j = 0; j < dim; j++) center[j] /= (double)npts;
        double semi = 0.0;
        for (int j = 0; j < dim; j++)
            for (int i = cs; i <= ce; i++) semi = std::max(semi, std::fabs(coord[j * n_point + i] - center[j]));
        semi += 1e-8;
        /* fixed-seed shift of the centre to break symmetric distributions */
        double shift_scale = semi * 1e-3;
        srand48(19241112);
        for (int j = 0; j < dim; j++) center[j] += (drand48() * 0.5 + 0.25) * shift_scale;
        semi = 0.0;
        for (int j = 0; j < dim; j++)
            for (int i = cs; i <= ce; i++) semi = std::max(semi, std::fabs(coord[j * n_point + i] - center[j]));
        semi += 1e-8;
        for (int j = 0; j < dim; j++) {
            enbox[j] = center[j] - semi - 2e-12;
            enbox[dim + j] = 2 * semi + 4e-12;
        }
    } else {
        std::memcpy(enbox, enbox_in, sizeof(enbox));
    }
    TreeNode *node = new TreeNode();
    if (npts <= max_leaf_points || enbox[dim] <= max_leaf_size) {
        node->pt_s = cs; node->pt_e = ce;
        node->po_idx = pv.curr_po_idx++;
        node->level = level;
        std::memcpy(node->enbox, enbox, sizeof(enbox));
        pv.n_leaf++;
        return node;
    }
    std::vector<int> rel(npts * dim), cid(npts, 0);
    int pow2 = 1;
    for (int j = 0; j < dim; j++) {
        for (int i = 0; i < npts; i++) {
            double r = coord[j * n_point + cs + i] - enbox[j];
            int v = (int)std::floor(2.0 * r / enbox[dim + j]);
            if (v == 2) v = 1;
            rel[j * npts + i] = v;
            cid[i] += v * pow2;
        }
        pow2 *= 2;
    }
    int sub_rel[8 * 3], sub_n[8] = {0}, displ[9];
    for (int i = 0; i < npts; i++) {
        sub_n[cid[i]]++;
        for (int j = 0; j < dim; j++) sub_rel[j * 8 + cid[i]] = rel[j * npts + i];
    }
    displ[0] = 0;
    for (int i = 1; i <= 8; i++) displ[i] = displ[i - 1] + sub_n[i - 1];
    for (int j = 0; j < dim; j++)
        std::memcpy(coord_tmp + j * n_point + cs, coord + j * n_point + cs, sizeof(double) * npts);
    std::memcpy(cidx_tmp + cs, cidx + cs, sizeof(int) * npts);
    for (int i = 0; i < npts; i++) {
        int dst = cs + displ[cid[i]]++;
        for (int j = 0; j < dim; j++) coord[j * n_point + dst] = coord_tmp[j * n_point + cs + i];
        cidx[dst] = cidx_tmp[cs + i];
    }
    displ[0] = 0;
    for (int i = 1; i <= 8; i++) displ[i] = displ[i - 1] + sub_n[i - 1];
    int nc = 0, n_node = 1, max_h = 0;
    for (int i = 0; i < 8; i++) {
        if (sub_n[i] == 0) continue;
        double sb[6];
        for (int j = 0; j < dim; j++) {
            sb[j] = enbox[j] + 0.5 * enbox[dim + j] * sub_rel[j * 8 + i] - 1e-12;
            sb[dim + j] = 0.5 * enbox[dim + j] + 2e-12;
        }
        TreeNode *c = bisect(level + 1, cs + displ[i], cs + displ[i + 1] - 1, n_point, max_leaf_size,
                             max_leaf_points, sb, coord, coord_tmp, cidx, cidx_tmp, pv);
        node->child[nc++] = c;
        n_node += c->n_node;
        max_h = std::max(max_h, c->height);
    }
    node->pt_s = cs; node->pt_e = ce;
    node->n_child = nc;
    node->n_node = n_node;
    node->po_idx = pv.curr_po_idx++;
    node->level = level;
    node->height = max_h + 1;
    std::memcpy(node->enbox, enbox, sizeof(enbox));
    return node;
}

void tree_to_array(const TreeNode *node, H2ERI_p h)
{
    for (int i = 0; i < node->n_child; i++) tree_to_array(node->child[i], h);
    int idx = node->po_idx;
    int *ch = h->children + idx * h->max_child;
    for (int i = 0; i < node->n_child; i++) {
        ch[i] = node->child[i]->po_idx;
        h->parent[node->child[i]->po_idx] = idx;
    }
    for (int i = node->n_child; i < h->max_child; i++) ch[i] = -1;
    h->pt_cluster[2 * idx] = node->pt_s;
    h->pt_cluster[2 * idx + 1] = node->pt_e;
    std::memcpy(h->enbox + idx * 6, node->enbox, sizeof(double) * 6);
    h->node_level[idx] = node->level;
    h->node_height[idx] = node->height;
    h->n_child[idx] = node->n_child;
    h->level_nodes[node->level * h->n_leaf_node + h->level_n_node[node->level]++] = idx;
    h->height_nodes[node->height * h->n_leaf_node + h->height_n_node[node->height]++] = idx;
}

bool box_admissible(const double *b0, const double *b1, double alpha)
{
    for (int i = 0; i < 3; i++) {
        double r0 = b0[3 + i], r1 = b1[3 + i];
        double c0 = b0[i] + 0.5 * r0, c1 = b1[i] + 0.5 * r1;
        if (std::fabs(c0 - c1) >= alpha * std::min(r0, r1) + 0.5 * (r0 + r1)) return true;
    }
    return false;
}

/* Reduced (in)admissible pairs, dual tree traversal
 * (src/H2ERI_partition_points.c:321-426). */
void reduced_pairs(H2ERI_p h, int n0, int n1, std::vector<int> &adm, std::vector<int> &inadm, int &min_adm_level)
{
    const int *nchild = h->n_child, *lvl = h->node_level;
    if (n0 == n1) {
        if (nchild[n0] == 0) return;
        const int *c = h->children + n0 * h->max_child;
        for (int i = 0; i < nchild[n0]; i++) reduced_pairs(h, c[i], c[i], adm, inadm, min_adm_level);
        for (int i = 0; i < nchild[n0]; i++)
            for (int j = i + 1; j < nchild[n0]; j++) reduced_pairs(h, c[i], c[j], adm, inadm, min_adm_level);
        return;
    }
    if (box_admissible(h->enbox + 6 * n0, h->enbox + 6 * n1, H2G_ALPHA_H2) &&
        lvl[n0] >= h->min_adm_level && lvl[n1] >= h->min_adm_level) {
        adm.push_back(n0);
        adm.push_back(n1);
        min_adm_level = std::min(min_adm_level, std::max(lvl[n0], lvl[n1]));
        return;
    }
    int c0 = nchild[n0], c1 = nchild[n1];
    if (c0 == 0 && c1 == 0) {
        inadm.push_back(n0);
        inadm.push_back(n1);
        return;
    }
    const int *ch0 = h->children + n0 * h->max_child, *ch1 = h->children + n1 * h->max_child;
    if (c0 == 0) {
        for (int j = 0; j < c1; j++) reduced_pairs(h, n0, ch1[j], adm, inadm, min_adm_level);
        return;
    }
    if (c1 == 0) {
        for (int i = 0; i < c0; i++) reduced_pairs(h, ch0[i], n1, adm, inadm, min_adm_level);
        return;
    }
    for (int i = 0; i < c0; i++)
        for (int j = 0; j < c1; j++) reduced_pairs(h, ch0[i], ch1[j], adm, inadm, min_adm_level);
}

void partition_points(H2ERI_p h, int n_point, const double *coord, int max_leaf_points, double max_leaf_size)
{
    double st = wtime();
    h->n_point = n_point;
    h->max_leaf_points = max_leaf_points;
    h->max_leaf_size = max_leaf_size;
    h->coord_idx = (int *)std::malloc(sizeof(int) * (size_t)n_point);
    h->coord = (double *)std::malloc(sizeof(double) * (size_t)n_point * 3);
    h->coord0 = (double *)std::malloc(sizeof(double) * (size_t)n_point * 3);
    std::memcpy(h->coord, coord, sizeof(double) * (size_t)n_point * 3);
    std::memcpy(h->coord0, coord, sizeof(double) * (size_t)n_point * 3);
    for (int i = 0; i < n_point; i++) h->coord_idx[i] = i;
    std::vector<int> cidx_tmp(n_point);
    std::vector<double> coord_tmp((size_t)n_point * 3);
    PartVars pv;
    TreeNode *root = bisect(0, 0, n_point - 1, n_point, max_leaf_size, max_leaf_points, nullptr, h->coord,
                            coord_tmp.data(), h->coord_idx, cidx_tmp.data(), pv);
    int n_node = root->n_node, nl = pv.max_level + 1;
    h->n_node = n_node;
    h->root_idx = n_node - 1;
    h->n_leaf_node = pv.n_leaf;
    h->max_level = pv.max_level;
    h->parent = (int *)std::malloc(sizeof(int) * n_node);
    h->children = (int *)std::malloc(sizeof(int) * n_node * h->max_child);
    h->pt_cluster = (int *)std::malloc(sizeof(int) * n_node * 2);
    h->mat_cluster = (int *)std::malloc(sizeof(int) * n_node * 2);
    h->n_child = (int *)std::malloc(sizeof(int) * n_node);
    h->node_level = (int *)std::malloc(sizeof(int) * n_node);
    h->node_height = (int *)std::malloc(sizeof(int) * n_node);
    h->level_n_node = (int *)std::calloc(nl, sizeof(int));
    h->level_nodes = (int *)std::malloc(sizeof(int) * nl * h->n_leaf_node);
    h->height_n_node = (int *)std::calloc(nl, sizeof(int));
    h->height_nodes = (int *)std::malloc(sizeof(int) * nl * h->n_leaf_node);
    h->enbox = (double *)std::malloc(sizeof(double) * n_node * 6);
    tree_to_array(root, h);
    h->parent[h->root_idx] = -1;
    delete root;

    h->min_adm_level = 0;
    int min_adm = h->max_level;
    std::vector<int> adm, inadm;
    reduced_pairs(h, h->root_idx, h->root_idx, adm, inadm, min_adm);
    h->min_adm_level = min_adm;
    h->n_r_adm_pair = (int)adm.size() / 2;
    h->n_r_inadm_pair = (int)inadm.size() / 2;
    h->r_adm_pairs = (int *)std::malloc(sizeof(int) * std::max<size_t>(adm.size(), 1));
    h->r_inadm_pairs = (int *)std::malloc(sizeof(int) * std::max<size_t>(inadm.size(), 1));
    if (!adm.empty()) std::memcpy(h->r_adm_pairs, adm.data(), sizeof(int) * adm.size());
    if (!inadm.empty()) std::memcpy(h->r_inadm_pairs, inadm.data(), sizeof(int) * inadm.size());
    h->timers[PT_TIMER_IDX] = wtime() - st;
}

}  // namespace

extern "C" void H2ERI_partition(H2ERI_p h)
{
    const int num_sp = h->num_sp;
    H2G_CHECK(num_sp > 0, "H2ERI_partition: no screened shell pairs (call H2ERI_process_shells first)\n");
    /* 1. partition SSP centres (src/H2ERI_partition.c:28-98) */
    int nbfp_total = 0;
    for (int i = 0; i < num_sp; i++) nbfp_total += NCART(h->sp_shells[i].am) * NCART(h->sp_shells[i + num_sp].am);
    h->krnl_mat_size = nbfp_total;
    partition_points(h, num_sp, h->sp_center, 300, 1.0);
    std::memcpy(h->sp_center, h->coord, sizeof(double) * 3 * (size_t)num_sp);
    {
        shell_t *sh_new = (shell_t *)std::calloc((size_t)num_sp * 2, sizeof(shell_t));
        double *ext_new = (double *)std::malloc(sizeof(double) * (size_t)num_sp);
        int *idx_new = (int *)std::malloc(sizeof(int) * (size_t)num_sp * 2);
        for (int i = 0; i < num_sp; i++) {
            int c = h->coord_idx[i];
            ext_new[i] = h->sp_extent[c];
            sh_new[i] = h->sp_shells[c];
            sh_new[i + num_sp] = h->sp_shells[c + num_sp];
            idx_new[i] = h->sp_shell_idx[c];
            idx_new[i + num_sp] = h->sp_shell_idx[c + num_sp];
        }
        std::free(h->sp_shells);   /* alpha/coef ownership moved to sh_new */
        std::free(h->sp_extent);
        std::free(h->sp_shell_idx);
        h->sp_shells = sh_new;
        h->sp_extent = ext_new;
        h->sp_shell_idx = idx_new;
    }
    /* shell pairs in (N, M) order: first shell is N = sp_shells[i + num_sp] */
    h->sp = (multi_sp_t *)std::calloc((size_t)num_sp, sizeof(multi_sp_t));
    h->index_seq = (int *)std::malloc(sizeof(int) * (size_t)num_sp);
    for (int i = 0; i < num_sp; i++) {
        h->index_seq[i] = i;
        h2g_shell N = as_h2g(&h->sp_shells[i + num_sp]), M = as_h2g(&h->sp_shells[i]);
        h2g_pair *pr = (h2g_pair *)std::malloc(sizeof(h2g_pair));
        h2g_pair_init(pr, &N, &M);
        h->sp[i].am1 = N.am;
        h->sp[i].am2 = M.am;
        h->sp[i].nprim = pr->nprim;
        h->sp[i].nshell12 = 1;
        h->sp[i].owns = 1;
        h->sp[i].capacity = 1;
        h->sp[i].pairs = (void **)std::malloc(sizeof(void *));
        h->sp[i].pairs[0] = pr;
    }

    /* 2. basis-function and bf-pair offsets (src/H2ERI_partition.c:108-143) */
    int nshell = h->nshell;
    h->shell_bf_sidx = (int *)std::malloc(sizeof(int) * (nshell + 1));
    h->sp_nbfp = (int *)std::malloc(sizeof(int) * num_sp);
    h->sp_bfp_sidx = (int *)std::malloc(sizeof(int) * (num_sp + 1));
    h->shell_bf_sidx[0] = 0;
    h->max_am = 0;
    for (int i = 0; i < nshell; i++) {
        h->shell_bf_sidx[i + 1] = h->shell_bf_sidx[i] + NCART(h->shells[i].am);
        h->max_am = std::max(h->max_am, h->shells[i].am);
    }
    h->num_bf = h->shell_bf_sidx[nshell];
    h->max_shell_nbf = NCART(h->max_am);
    h->sp_bfp_sidx[0] = 0;
    for (int i = 0; i < num_sp; i++) {
        int nbfp = NCART(h->sp_shells[i].am) * NCART(h->sp_shells[i + num_sp].am);
        h->sp_nbfp[i] = nbfp;
        h->sp_bfp_sidx[i + 1] = h->sp_bfp_sidx[i] + nbfp;
    }
    h->num_sp_bfp = h->sp_bfp_sidx[num_sp];

    /* 3. box extents (src/H2ERI_partition.c:152-226) */
    int n_node = h->n_node;
    h->box_extent = (double *)std::calloc((size_t)n_node, sizeof(double));
    /* the reference stops at level 1; the root is included here so that a
     * one-node tree (tiny molecule, root admissible level 0) has a defined extent */
    for (int lv = h->max_level; lv >= 0; lv--) {
        for (int j = 0; j < h->level_n_node[lv]; j++) {
            int node = h->level_nodes[lv * h->n_leaf_node + j];
            const double *eb = h->enbox + 6 * node;
            double ec[3] = {eb[0] + 0.5 * eb[3], eb[1] + 0.5 * eb[4], eb[2] + 0.5 * eb[5]};
            if (h->n_child[node] == 0) {
                double be = 0.0;
                for (int d = 0; d < 3; d++) {
                    const double *cd = h->sp_center + d * num_sp;
                    for (int k = h->pt_cluster[2 * node]; k <= h->pt_cluster[2 * node + 1]; k++) {
                        double t = 0.5 * eb[3 + d] - std::fabs(cd[k] - ec[d]);
                        t = (h->sp_extent[k] - t) / eb[3 + d];
                        be = std::max(be, std::max(t, 0.1));
                    }
                }
                h->box_extent[node] = std::ceil(be);
            } else {
                double be = 0.0;
                for (int k = 0; k < h->n_child[node]; k++)
                    be = std::max(be, h->box_extent[h->children[node * h->max_child + k]]);
                h->box_extent[node] = std::ceil(0.5 * be);
            }
        }
    }

    /* 4. vector ranges of nodes (src/H2ERI_partition.c:233-265) */
    int off = 0;
    for (int i = 0; i < n_node; i++) {
        if (h->n_child[i] == 0) {
            int nb = h->sp_bfp_sidx[h->pt_cluster[2 * i + 1] + 1] - h->sp_bfp_sidx[h->pt_cluster[2 * i]];
            h->mat_cluster[2 * i] = off;
            h->mat_cluster[2 * i + 1] = off + nb - 1;
            off += nb;
        } else {
            const int *c = h->children + i * h->max_child;
            h->mat_cluster[2 * i] = h->mat_cluster[2 * c[0]];
            h->mat_cluster[2 * i + 1] = h->mat_cluster[2 * c[h->n_child[i] - 1] + 1];
        }
    }

    /* 5. per-node admissible / inadmissible partner lists (src/H2ERI_partition.c:273-360) */
    {
        const int *leaf = h->height_nodes;
        std::vector<std::vector<int>> adm(n_node), inadm(n_node);
        for (int i = 0; i < h->n_r_adm_pair; i++) {
            int a = h->r_adm_pairs[2 * i], b = h->r_adm_pairs[2 * i + 1];
            adm[a].push_back(b);
            adm[b].push_back(a);
        }
        for (int i = 0; i < h->n_leaf_node; i++) inadm[leaf[i]].push_back(leaf[i]);
        for (int i = 0; i < h->n_r_inadm_pair; i++) {
            int a = h->r_inadm_pairs[2 * i], b = h->r_inadm_pairs[2 * i + 1];
            inadm[a].push_back(b);
            inadm[b].push_back(a);
        }
        /* the reference fills the CSR with leaf self pairs first, then pairs in list order */
        auto to_csr = [&](std::vector<std::vector<int>> &lists, int **sidx, int **vals) {
            *sidx = (int *)std::malloc(sizeof(int) * (n_node + 1));
            size_t tot = 0;
            for (auto &l : lists) tot += l.size();
            *vals = (int *)std::malloc(sizeof(int) * std::max<size_t>(tot, 1));
            (*sidx)[0] = 0;
            for (int i = 0; i < n_node; i++) {
                if (!lists[i].empty())
                    std::memcpy(*vals + (*sidx)[i], lists[i].data(), sizeof(int) * lists[i].size());
                (*sidx)[i + 1] = (*sidx)[i] + (int)lists[i].size();
            }
        };
        to_csr(adm, &h->node_adm_pairs_sidx, &h->node_adm_pairs);
        to_csr(inadm, &h->node_inadm_pairs_sidx, &h->node_inadm_pairs);
    }

    /* 6. per-shell partner lists for K (src/H2ERI_partition.c:371-427) */
    {
        std::vector<std::vector<std::pair<int, int>>> pl(nshell);
        for (int i = 0; i < num_sp; i++) {
            int s0 = h->sp_shell_idx[i], s1 = h->sp_shell_idx[i + num_sp];
            pl[s0].push_back({s1, i});
            if (s0 != s1) pl[s1].push_back({s0, i});
        }
        h->plist_sidx = (int *)std::malloc(sizeof(int) * (nshell + 1));
        h->plist = (int *)std::malloc(sizeof(int) * 2 * (size_t)num_sp);
        h->plist_idx = (int *)std::malloc(sizeof(int) * 2 * (size_t)num_sp);
        h->plist_sidx[0] = 0;
        for (int s = 0; s < nshell; s++) {
            std::sort(pl[s].begin(), pl[s].end());
            int base = h->plist_sidx[s];
            for (size_t k = 0; k < pl[s].size(); k++) {
                h->plist[base + k] = pl[s][k].first;
                h->plist_idx[base + k] = pl[s][k].second;
            }
            h->plist_sidx[s + 1] = base + (int)pl[s].size();
        }
    }

    /* 7. per-thread buffers */
    h->thread_buffs = (H2E_thread_buf_p *)std::malloc(sizeof(H2E_thread_buf_p) * h->n_thread);
    for (int i = 0; i < h->n_thread; i++) h->thread_buffs[i] = tbuf_new(h->krnl_mat_size);
}
