/*
 * Electron-repulsion integral blocks on the GPU, for the per-geometry set-up
 * of the near-field (D) and coupling (B) blocks.
 *
 * The reference evaluates these blocks on the host through SIMINT
 * (H2P-ERI src/CMS.c:387-451, called from src/H2ERI_build_H2.c:910-1403).
 * This file evaluates the same shell quartets (NM|QP) with the recurrences
 * of the host engine (h2g_ints.c): Obara-Saika vertical recurrence per
 * primitive quartet, contraction, then the Head-Gordon-Pople horizontal
 * recurrence on the bra and on the ket (S. Obara, A. Saika, J. Chem. Phys.
 * 84, 3963 (1986); M. Head-Gordon, J. A. Pople, J. Chem. Phys. 89, 5777
 * (1988)). The component tables and the Boys-function grid are the host
 * engine's own (h2g_ints_tables), so both give the same integrals up to
 * the order of floating-point sums.
 *
 * Work: one warp per shell quartet. Quartet classes (angular momenta) are
 * launched separately, each with its own shared-memory workspace per warp.
 * For a class with a small recurrence table and many primitive quartets the
 * lanes take primitive quartets (each lane its own table); otherwise the
 * warp builds one primitive quartet's table at a time, lanes over the
 * table's (component, order) entries. The vertical-recurrence table is
 * compact: entry [e|f]^(m) exists for m <= M - |e| - |f|.
 *
 * Shells up to d (the cc-pVDZ basis of this package's workloads); a
 * structure with higher angular momentum stays on the host engine.
 */
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "h2g_eri.h"
#include "h2g_gpu_api.h"
#include "h2g_ints.h"

namespace h2g {
namespace eri {

constexpr int kMaxAm = 2;                       /* per shell on the GPU  */
constexpr int kMaxL = 2 * H2G_MAX_AM;           /* host engine's tables   */
constexpr int kMaxCum = (kMaxL + 1) * (kMaxL + 2) * (kMaxL + 3) / 6;
constexpr int kBoysGrid = 801, kBoysTab = 4 * H2G_MAX_AM + 1 + 7 + 1;
constexpr double kBoysH = 0.05, kBoysTmax = 40.0;
constexpr int kWarps = 4;                       /* warps per CTA (at most) */

__constant__ int c_lxyz[kMaxCum][3];
__constant__ int c_cum[kMaxL + 2];
__constant__ int c_dir[kMaxCum], c_prev[kMaxCum], c_prev2[kMaxCum];
__constant__ int c_minus[kMaxCum][3], c_plus[kMaxCum][3];

__host__ __device__ inline int ncart(int l) { return (l + 1) * (l + 2) / 2; }
__host__ __device__ inline int ncum(int l) { return (l + 1) * (l + 2) * (l + 3) / 6; }

/* One screened shell pair (N, M): angular momenta, centres, and its
 * primitive pairs [poff, poff + nprim) in the primitive arrays. */
struct Ssp {
    int am1, am2, nprim, poff;
    double A[3], B[3];
};

/* One shell quartet: bra and ket pairs, and where its nr x nc block goes in
 * the output (element (r, c) at off + r ld + c, and at off_t + c ld + r if
 * off_t >= 0). */
struct Task {
    int bra, ket;
    long long off, off_t;
    int ld, pad_;
};

/* Per-class constants and workspace layout (doubles per warp). */
struct Cls {
    int la, lb, lc, ld, La, Lc, M, ne, nf;
    int T;        /* compact table size                          */
    int A;        /* contracted [e|f] entries for the HRR        */
    int lvl;      /* largest HRR level array                     */
    int lane_ok;  /* lanes may take primitive quartets           */
    int lstride;  /* doubles per lane in lane mode (odd: no bank conflicts between lanes) */
    int ws;       /* workspace doubles per warp                  */
    const int *voff;   /* compact offsets [ne * nf] (device)     */
};

/* Boys function F_0..F_mmax(T): the host engine's grid with a 7-term
 * Taylor step below T = 40, the asymptotic form with upward recursion
 * above it (same formulas as h2g_boys). */
__device__ void boys(int mmax, double T, const double *__restrict__ tab, double *F)
{
    if (T < kBoysTmax) {
        const int k = (int)(T / kBoysH + 0.5);
        const double d = T - k * kBoysH;
        const double *row = tab + (size_t)k * kBoysTab;
        const double inv_fact[7] = {1.0, 1.0, 1.0 / 2, 1.0 / 6, 1.0 / 24, 1.0 / 120, 1.0 / 720};
        double f[7], pw = 1.0;
#pragma unroll
        for (int j = 0; j < 7; j++) {
            f[j] = pw * inv_fact[j];
            pw *= -d;
        }
        for (int m = 0; m <= mmax; m++) {
            double s = 0.0;
#pragma unroll
            for (int j = 0; j < 7; j++) s += __ldg(row + m + j) * f[j];
            F[m] = s;
        }
    } else {
        const double et = exp(-T), inv2t = 0.5 / T;
        F[0] = 0.5 * sqrt(M_PI / T);
        for (int m = 0; m < mmax; m++) F[m + 1] = ((2 * m + 1) * F[m] - et) * inv2t;
    }
}

/* F_m(T) for one order m and T < 40: the same grid and Taylor step as boys(). */
__device__ double boys_one(int m, double T, const double *__restrict__ tab)
{
    const int k = (int)(T / kBoysH + 0.5);
    const double d = T - k * kBoysH;
    const double *row = tab + (size_t)k * kBoysTab + m;
    const double inv_fact[7] = {1.0, 1.0, 1.0 / 2, 1.0 / 6, 1.0 / 24, 1.0 / 120, 1.0 / 720};
    double pw = 1.0, s = 0.0;
#pragma unroll
    for (int j = 0; j < 7; j++) {
        s += __ldg(row + j) * (pw * inv_fact[j]);
        pw *= -d;
    }
    return s;
}

/* Scalars of one primitive quartet (p from the bra pair, q from the ket). */
struct Prim {
    double PA[3], WP[3], WQ[3], QC[3];
    double i2p, rp, i2q, rq, i2pq, pref, T;
};

__device__ inline void prim_setup(const Ssp &bra, const Ssp &ket, int i, int j, const double *__restrict__ P,
                                  const double *__restrict__ pe, const double *__restrict__ K,
                                  const double *__restrict__ ip, Prim &q)
{
    const int bi = bra.poff + i, kj = ket.poff + j;
    const double p = pe[bi], qq = pe[kj];
    const double ipq = 1.0 / (p + qq), rho = p * qq * ipq;
    double PQ2 = 0.0;
#pragma unroll
    for (int d = 0; d < 3; d++) {
        const double pd = P[3 * bi + d], qd = P[3 * kj + d], pq = pd - qd;
        q.PA[d] = pd - bra.A[d];
        q.WP[d] = -(qq * ipq) * pq;
        q.WQ[d] = (p * ipq) * pq;
        q.QC[d] = qd - ket.A[d];
        PQ2 += pq * pq;
    }
    q.i2p = 0.5 * ip[bi];
    q.rp = qq * ipq;
    q.i2q = 0.5 * ip[kj];
    q.rq = p * ipq;
    q.i2pq = 0.5 * ipq;
    q.T = rho * PQ2;
    q.pref = 34.986836655249725 /* 2 pi^2.5 */ * K[bi] * ip[bi] * (K[kj] * ip[kj]) * sqrt(ipq);
}

__device__ inline int lsum(int c) { return c_lxyz[c][0] + c_lxyz[c][1] + c_lxyz[c][2]; }

/* Vertical recurrence of one primitive quartet into V (compact layout), by
 * one thread (lane mode). V[voff[0] + m] = pref F_m already set. */
__device__ void vrr_serial(const Cls &C, const Prim &q, double *V)
{
    const int *voff = C.voff;
    const int ne = C.ne, nf = C.nf, M = C.M;
    for (int c = 1; c < ne; c++) {
        const int L = lsum(c), d = c_dir[c], e = c_prev[c], e2 = c_prev2[c];
        double *vc = V + voff[c * nf];
        const double *ve = V + voff[e * nf];
        if (e2 >= 0) {
            const double *ve2 = V + voff[e2 * nf];
            const double ei2p = (double)(c_lxyz[c][d] - 1) * q.i2p;
            for (int m = 0; m <= M - L; m++)
                vc[m] = q.PA[d] * ve[m] + q.WP[d] * ve[m + 1] + ei2p * (ve2[m] - q.rp * ve2[m + 1]);
        } else {
            for (int m = 0; m <= M - L; m++) vc[m] = q.PA[d] * ve[m] + q.WP[d] * ve[m + 1];
        }
    }
    for (int c = 1; c < nf; c++) {
        const int Lf = lsum(c), d = c_dir[c], f = c_prev[c], f2 = c_prev2[c];
        const double fi2q = (double)(c_lxyz[c][d] - 1) * q.i2q;
        for (int e = 0; e < ne; e++) {
            const int Le = lsum(e), mmax = M - Le - Lf;
            if (mmax < 0) continue;
            double *vc = V + voff[e * nf + c];
            const double *vf = V + voff[e * nf + f];
            const double *vf2 = f2 >= 0 ? V + voff[e * nf + f2] : nullptr;
            const int em = c_minus[e][d];
            const double *vem = em >= 0 ? V + voff[em * nf + f] : nullptr;
            const double ed2pq = (double)c_lxyz[e][d] * q.i2pq;
            for (int m = 0; m <= mmax; m++) {
                double v = q.QC[d] * vf[m] + q.WQ[d] * vf[m + 1];
                if (vf2) v += fi2q * (vf2[m] - q.rq * vf2[m + 1]);
                if (vem) v += ed2pq * vem[m + 1];
                vc[m] = v;
            }
        }
    }
}

/* The same by a warp: lanes over the orders m (bra side) and over the
 * (e, m) entries of one ket component (ket side). */
__device__ void vrr_warp(const Cls &C, const Prim &q, double *V, int lane)
{
    const int *voff = C.voff;
    const int ne = C.ne, nf = C.nf, M = C.M, nm = M + 1;
    for (int c = 1; c < ne; c++) {
        const int L = lsum(c), d = c_dir[c], e = c_prev[c], e2 = c_prev2[c];
        const int m = lane;
        if (m <= M - L) {
            double *vc = V + voff[c * nf];
            const double *ve = V + voff[e * nf];
            double v = q.PA[d] * ve[m] + q.WP[d] * ve[m + 1];
            if (e2 >= 0) {
                const double *ve2 = V + voff[e2 * nf];
                v += (double)(c_lxyz[c][d] - 1) * q.i2p * (ve2[m] - q.rp * ve2[m + 1]);
            }
            vc[m] = v;
        }
        __syncwarp();
    }
    for (int c = 1; c < nf; c++) {
        const int Lf = lsum(c), d = c_dir[c], f = c_prev[c], f2 = c_prev2[c];
        const double fi2q = (double)(c_lxyz[c][d] - 1) * q.i2q;
        for (int k = lane; k < ne * nm; k += 32) {
            const int e = k / nm, m = k - e * nm;
            const int Le = lsum(e);
            if (m > M - Le - Lf) continue;
            const double *vf = V + voff[e * nf + f];
            double v = q.QC[d] * vf[m] + q.WQ[d] * vf[m + 1];
            if (f2 >= 0) {
                const double *vf2 = V + voff[e * nf + f2];
                v += fi2q * (vf2[m] - q.rq * vf2[m + 1]);
            }
            const int em = c_minus[e][d];
            if (em >= 0) v += (double)c_lxyz[e][d] * q.i2pq * V[voff[em * nf + f] + m + 1];
            V[voff[e * nf + c] + m] = v;
        }
        __syncwarp();
    }
}

/* Horizontal recurrence by a warp, moving l2 units of angular momentum to
 * the second index of a pair: (a, b + 1_i| = (a + 1_i, b| + AB_i (a, b|.
 * src[(e - cum[l1]) * nrep + r] for |e| in [l1, l1 + l2]; the result
 * (a, b) for |a| = l1, |b| = l2 goes to dst[(ia * nb + ib) * nrep + r], or
 * with `tr` to dst[r * (na nb) + ia * nb + ib]. b0, b1: level buffers. */
__device__ void hrr_warp(int l1, int l2, const double AB[3], const double *src, int nrep, double *dst, bool tr,
                         double *b0, double *b1, int lane)
{
    const int na = ncart(l1), nb = ncart(l2), e0 = c_cum[l1];
    const double *cur = src;
    int nbp = 1;
    for (int j = 1; j <= l2; j++) {
        const int nbj = ncart(j), emax = c_cum[l1 + l2 - j + 1];
        double *nxt = (j & 1) ? b0 : b1;
        const int nent = (emax - e0) * nbj * nrep;
        for (int k = lane; k < nent; k += 32) {
            const int r = k % nrep, t = k / nrep, ib = t % nbj, e = e0 + t / nbj;
            const int bf = c_cum[j] + ib, d = c_dir[bf], bp = c_prev[bf] - c_cum[j - 1];
            const int ep = c_plus[e][d];
            nxt[k] = cur[((ep - e0) * nbp + bp) * nrep + r] + AB[d] * cur[((e - e0) * nbp + bp) * nrep + r];
        }
        __syncwarp();
        cur = nxt;
        nbp = nbj;
    }
    const int nab = na * nb;
    for (int k = lane; k < nab * nrep; k += 32) {
        const int r = k % nrep, ab = k / nrep;
        const double v = cur[ab * nrep + r];   /* level l2 rows: a in [0, na), b in [0, nb) */
        if (tr) dst[r * nab + ab] = v;
        else dst[ab * nrep + r] = v;
    }
    __syncwarp();
}

/* One class of quartets: warp w of the grid takes tasks w, w + W, ... */
__global__ void __launch_bounds__(32 * kWarps) k_eri(Cls C, const Task *__restrict__ tasks, int n_task,
                                                     const Ssp *__restrict__ ssp, const double *__restrict__ P,
                                                     const double *__restrict__ pe, const double *__restrict__ K,
                                                     const double *__restrict__ ip,
                                                     const double *__restrict__ boys_tab, double *__restrict__ out)
{
    extern __shared__ double smem[];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    double *ws = smem + (size_t)wib * C.ws;
    double *acc = ws, *scr = ws + C.A;
    const int nwarp = gridDim.x * (blockDim.x >> 5);
    const int nfa = C.nf - c_cum[C.lc];
    const int e0 = c_cum[C.la], f0 = c_cum[C.lc];
    const int nA = ncart(C.la), nB = ncart(C.lb), nC = ncart(C.lc), nD = ncart(C.ld);
    const int nab = nA * nB, ncd = nC * nD;
    for (int ti = blockIdx.x * (blockDim.x >> 5) + wib; ti < n_task; ti += nwarp) {
        const Task tk = tasks[ti];
        const Ssp bra = ssp[tk.bra], ket = ssp[tk.ket];
        const int nk = ket.nprim, nq = bra.nprim * nk;
        for (int a = lane; a < C.A; a += 32) acc[a] = 0.0;
        __syncwarp();
        if (C.lane_ok && nq >= 8) {
            /* lanes over primitive quartets, each with its own table and sums */
            double *V = scr + (size_t)lane * C.lstride;
            double *la = V + C.T;
            for (int a = 0; a < C.A; a++) la[a] = 0.0;
            for (int qi = lane; qi < nq; qi += 32) {
                Prim q;
                prim_setup(bra, ket, qi / nk, qi % nk, P, pe, K, ip, q);
                double F[4 * kMaxAm + 1];
                boys(C.M, q.T, boys_tab, F);
                for (int m = 0; m <= C.M; m++) V[m] = q.pref * F[m];
                vrr_serial(C, q, V);
                for (int e = e0; e < C.ne; e++)
                    for (int f = f0; f < C.nf; f++) la[(e - e0) * nfa + (f - f0)] += V[C.voff[e * C.nf + f]];
            }
            __syncwarp();
            for (int a = lane; a < C.A; a += 32) {
                double s = 0.0;
                for (int l = 0; l < 32; l++) s += scr[(size_t)l * C.lstride + C.T + a];
                acc[a] = s;
            }
            __syncwarp();
        } else {
            /* the warp on one primitive quartet at a time */
            double *V = scr;
            for (int qi = 0; qi < nq; qi++) {
                Prim q;
                prim_setup(bra, ket, qi / nk, qi % nk, P, pe, K, ip, q);
                if (q.T < kBoysTmax) {
                    if (lane <= C.M) V[lane] = q.pref * boys_one(lane, q.T, boys_tab);   /* one order per lane */
                } else if (lane == 0) {
                    double F[4 * kMaxAm + 1];
                    boys(C.M, q.T, boys_tab, F);
                    for (int m = 0; m <= C.M; m++) V[m] = q.pref * F[m];
                }
                __syncwarp();
                vrr_warp(C, q, V, lane);
                for (int a = lane; a < C.A; a += 32) {
                    const int e = e0 + a / nfa, f = f0 + a % nfa;
                    acc[a] += V[C.voff[e * C.nf + f]];
                }
                __syncwarp();
            }
        }
        /* HRR: bra (a, b) with the ket entries trailing, written transposed so
         * that the ket HRR runs with (a, b) trailing */
        const double AB[3] = {bra.A[0] - bra.B[0], bra.A[1] - bra.B[1], bra.A[2] - bra.B[2]};
        const double CD[3] = {ket.A[0] - ket.B[0], ket.A[1] - ket.B[1], ket.A[2] - ket.B[2]};
        /* scratch after the sums: X, two level buffers, R (lvl doubles each) */
        double *X = scr, *b0 = scr + C.lvl, *b1 = scr + 2 * C.lvl, *R = scr + 3 * C.lvl;
        hrr_warp(C.la, C.lb, AB, acc, nfa, X, true, b0, b1, lane);   /* X[f'][ab]                  */
        hrr_warp(C.lc, C.ld, CD, X, nab, R, false, b0, b1, lane);    /* R[(ic nD + id) nab + ab]   */
        for (int k = lane; k < nab * ncd; k += 32) {
            const int ab = k / ncd, cd = k - ab * ncd;
            const double v = R[cd * nab + ab];
            out[tk.off + (long long)ab * tk.ld + cd] = v;
            if (tk.off_t >= 0) out[tk.off_t + (long long)cd * tk.ld + ab] = v;
        }
        __syncwarp();
    }
}

/* ---- host side ---- */

struct Tables {
    bool ok = false;
    int device = -1;
    double *boys = nullptr;
    std::vector<int> lxyz, cum, dir, prev, prev2, minus, plus;
};

std::mutex g_mu;
std::map<int, Tables> g_tab;   /* per device */

int ensure_tables(Tables **out)
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) { set_error("gpu eri: no device"); return 9; }
    std::lock_guard<std::mutex> lk(g_mu);
    Tables &t = g_tab[dev];
    if (!t.ok) {
        int dims[4];
        h2g_ints_tables(nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, dims);
        if (dims[0] != kMaxL || dims[1] != kMaxCum || dims[2] != kBoysGrid || dims[3] != kBoysTab) {
            set_error("gpu eri: table shapes differ from the host engine's");
            return 3;
        }
        t.lxyz.resize(kMaxCum * 3); t.cum.resize(kMaxL + 2); t.dir.resize(kMaxCum); t.prev.resize(kMaxCum);
        t.prev2.resize(kMaxCum); t.minus.resize(kMaxCum * 3); t.plus.resize(kMaxCum * 3);
        std::vector<double> boys((size_t)kBoysGrid * kBoysTab);
        h2g_ints_tables(t.lxyz.data(), t.cum.data(), t.dir.data(), t.prev.data(), t.prev2.data(), t.minus.data(),
                        t.plus.data(), boys.data(), dims);
        if (cudaMemcpyToSymbol(c_lxyz, t.lxyz.data(), sizeof(int) * kMaxCum * 3) != cudaSuccess ||
            cudaMemcpyToSymbol(c_cum, t.cum.data(), sizeof(int) * (kMaxL + 2)) != cudaSuccess ||
            cudaMemcpyToSymbol(c_dir, t.dir.data(), sizeof(int) * kMaxCum) != cudaSuccess ||
            cudaMemcpyToSymbol(c_prev, t.prev.data(), sizeof(int) * kMaxCum) != cudaSuccess ||
            cudaMemcpyToSymbol(c_prev2, t.prev2.data(), sizeof(int) * kMaxCum) != cudaSuccess ||
            cudaMemcpyToSymbol(c_minus, t.minus.data(), sizeof(int) * kMaxCum * 3) != cudaSuccess ||
            cudaMemcpyToSymbol(c_plus, t.plus.data(), sizeof(int) * kMaxCum * 3) != cudaSuccess) {
            set_error("gpu eri: constant tables not copied");
            return 10;
        }
        if (cudaMalloc(&t.boys, boys.size() * sizeof(double)) != cudaSuccess ||
            cudaMemcpy(t.boys, boys.data(), boys.size() * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess) {
            set_error("gpu eri: Boys table not copied");
            return 10;
        }
        t.device = dev;
        t.ok = true;
    }
    *out = &t;
    return 0;
}

/* Class constants on the host, with the compact table offsets. */
Cls make_class(const Tables &t, int la, int lb, int lc, int ld, std::vector<int> &voff)
{
    Cls C;
    std::memset(&C, 0, sizeof(C));
    C.la = la; C.lb = lb; C.lc = lc; C.ld = ld;
    C.La = la + lb; C.Lc = lc + ld; C.M = C.La + C.Lc;
    C.ne = ncum(C.La); C.nf = ncum(C.Lc);
    voff.assign((size_t)C.ne * C.nf, -1);
    auto L = [&](int c) { return t.lxyz[3 * c] + t.lxyz[3 * c + 1] + t.lxyz[3 * c + 2]; };
    int n = 0;
    for (int e = 0; e < C.ne; e++)
        for (int f = 0; f < C.nf; f++) {
            const int k = C.M - L(e) - L(f) + 1;
            /* every entry gets a slot (entries with k <= 0 are never read) */
            voff[(size_t)e * C.nf + f] = n;
            n += std::max(k, 1);
        }
    C.T = n;
    const int e0 = t.cum[la], f0 = t.cum[lc];
    C.A = (C.ne - e0) * (C.nf - f0);
    /* HRR levels: bra with nrep = nfa, then ket with nrep = nab */
    const int nfa = C.nf - f0, nab = ncart(la) * ncart(lb);
    int lvl = 0;
    for (int j = 1; j <= lb; j++) lvl = std::max(lvl, (t.cum[la + lb - j + 1] - e0) * ncart(j) * nfa);
    lvl = std::max(lvl, nfa * nab);   /* X */
    for (int j = 1; j <= ld; j++) lvl = std::max(lvl, (t.cum[lc + ld - j + 1] - f0) * ncart(j) * nab);
    lvl = std::max(lvl, nab * ncart(lc) * ncart(ld));   /* R */
    C.lvl = lvl;
    C.lstride = (C.T + C.A) | 1;
    const int lane_need = 32 * C.lstride;
    C.lane_ok = lane_need <= 20480;   /* 160 KB per warp at most */
    C.ws = C.A + std::max({C.lane_ok ? lane_need : 0, C.T, 4 * lvl});
    return C;
}

}  // namespace eri

using namespace eri;

/* Device state of one structure's shell pairs for the set-up. */
struct EriSet {
    int device = 0;   /* the device the shell pairs live on (set in every calling thread) */
    Ssp *ssp = nullptr;
    double *P = nullptr, *pe = nullptr, *K = nullptr, *ip = nullptr;
    std::vector<Ssp> host;
    int n_sp = 0;
};

int gpu_eri_usable()
{
    const char *e = std::getenv("H2G_SETUP_GPU");
    if (e != nullptr && std::strcmp(e, "0") == 0) return 0;
    int n = 0;
    return cudaGetDeviceCount(&n) == cudaSuccess && n > 0;
}

void gpu_eri_free(EriSet *s)
{
    if (s == nullptr) return;
    cudaFree(s->ssp); cudaFree(s->P); cudaFree(s->pe); cudaFree(s->K); cudaFree(s->ip);
    delete s;
}

int gpu_eri_create(int n_sp, const h2g_pair *const *pairs, EriSet **out)
{
    *out = nullptr;
    Tables *t;
    int rc = ensure_tables(&t);
    if (rc) return rc;
    EriSet *s = new EriSet();
    s->n_sp = n_sp;
    cudaGetDevice(&s->device);
    std::vector<double> P, pe, K, ip;
    for (int i = 0; i < n_sp; i++) {
        const h2g_pair *pr = pairs[i];
        if (pr->am1 > kMaxAm || pr->am2 > kMaxAm) {
            gpu_eri_free(s);
            set_error("gpu eri: shells above d are evaluated on the host");
            return 3;
        }
        Ssp q;
        q.am1 = pr->am1; q.am2 = pr->am2; q.nprim = pr->nprim; q.poff = (int)pe.size();
        for (int d = 0; d < 3; d++) { q.A[d] = pr->A[d]; q.B[d] = pr->B[d]; }
        for (int k = 0; k < pr->nprim; k++) {
            for (int d = 0; d < 3; d++) P.push_back(pr->P[3 * k + d]);
            pe.push_back(pr->p[k]);
            K.push_back(pr->K[k]);
            ip.push_back(pr->ip[k]);
        }
        s->host.push_back(q);
    }
    auto up = [&](auto **dst, const auto &v) {
        using T = typename std::remove_reference<decltype(v)>::type::value_type;
        if (cudaMalloc(dst, std::max<size_t>(v.size(), 1) * sizeof(T)) != cudaSuccess) return false;
        return v.empty() || cudaMemcpy(*dst, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice) == cudaSuccess;
    };
    if (!up(&s->ssp, s->host) || !up(&s->P, P) || !up(&s->pe, pe) || !up(&s->K, K) || !up(&s->ip, ip)) {
        gpu_eri_free(s);
        set_error("gpu eri: shell-pair upload failed");
        return 10;
    }
    *out = s;
    return 0;
}

/* Evaluate every quartet of every block request into one device buffer and
 * copy each block back to its host matrix. A request's block is
 * rows = the bf pairs of its bra pairs in order, columns = those of its ket
 * pairs (the layout of the host eri_pairs_to_mat); with `sym` (bra == ket,
 * a diagonal block) only quartets with bra index <= ket index are evaluated
 * and mirrored. */
static int eri_blocks_range(EriSet *s, Tables *t, EriReq *reqs_begin, size_t n_req);

int gpu_eri_blocks(EriSet *s, std::vector<EriReq> &reqs)
{
    if (cudaSetDevice(s->device) != cudaSuccess) {
        set_error("gpu eri: cannot select the device of the shell pairs");
        return 10;
    }
    Tables *t;
    int rc = ensure_tables(&t);
    if (rc) return rc;
    /* requests in groups of at most 2^27 output doubles (1 GB) on the device */
    auto nbfp = [&](int sp) { return ncart(s->host[sp].am1) * ncart(s->host[sp].am2); };
    size_t i = 0;
    while (i < reqs.size()) {
        size_t j = i;
        long long tot = 0;
        while (j < reqs.size()) {
            long long nr = 0, ncl = 0;
            for (int b : reqs[j].bra) nr += nbfp(b);
            for (int k : reqs[j].ket) ncl += nbfp(k);
            if (j > i && tot + nr * ncl > (1LL << 27)) break;
            tot += nr * ncl;
            j++;
        }
        rc = eri_blocks_range(s, t, reqs.data() + i, j - i);
        if (rc) return rc;
        i = j;
    }
    return 0;
}

/* One block of quartets in a device buffer: rows = bf pairs of bra[0..nbra),
 * columns = those of ket[0..nket), element (r, c) at off + r * ld + c; with
 * sym only quartets with bra position <= ket position, mirrored. */
struct BlockSpec {
    const int *bra, *ket;
    int nbra, nket;
    bool sym;
    long long off;
    int ld;
};

/* Evaluate the quartets of blocks into dout (device): one launch per quartet
 * class, classes on round-robin streams in order of decreasing work (so
 * that the small classes run beside the large ones); returns after the
 * kernels end. kms gets the milliseconds of the launches. */
static int launch_eri(EriSet *s, Tables *t, const std::vector<BlockSpec> &blocks, double *dout, double *kms)
{
    const int nc = kMaxAm + 1;
    std::vector<std::vector<Task>> by_cls((size_t)nc * nc * nc * nc);
    auto nbfp = [&](int sp) { return ncart(s->host[sp].am1) * ncart(s->host[sp].am2); };
    for (const BlockSpec &q : blocks) {
        int row = 0;
        for (int i = 0; i < q.nbra; i++) {
            const int b = q.bra[i];
            int col = 0;
            for (int j = 0; j < q.nket; j++) {
                const int k = q.ket[j];
                if (!q.sym || i <= j) {
                    Task tk;
                    tk.bra = b;
                    tk.ket = k;
                    tk.off = q.off + (long long)row * q.ld + col;
                    tk.off_t = (q.sym && i < j) ? q.off + (long long)col * q.ld + row : -1;
                    tk.ld = q.ld;
                    tk.pad_ = 0;
                    const Ssp &B = s->host[b], &Kt = s->host[k];
                    by_cls[((B.am1 * nc + B.am2) * nc + Kt.am1) * nc + Kt.am2].push_back(tk);
                }
                col += nbfp(k);
            }
            row += nbfp(b);
        }
    }
    *kms = 0.0;
    /* every class's tasks and table offsets in one upload */
    std::vector<Task> all_tasks;
    std::vector<int> all_voff;
    struct Launch { Cls C; size_t t0, nt; int warps; };
    std::vector<Launch> launches;
    size_t smem_need = 0;
    int dev = 0, smem_max = 0, n_sm = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&smem_max, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev);
    std::vector<size_t> voff_at;
    for (int la = 0; la < nc; la++)
        for (int lb = 0; lb < nc; lb++)
            for (int lc = 0; lc < nc; lc++)
                for (int ld = 0; ld < nc; ld++) {
                    std::vector<Task> &v = by_cls[((la * nc + lb) * nc + lc) * nc + ld];
                    if (v.empty()) continue;
                    std::vector<int> voff;
                    Launch L;
                    L.C = make_class(*t, la, lb, lc, ld, voff);
                    const size_t ws_bytes = (size_t)L.C.ws * sizeof(double);
                    L.warps = (int)std::min<size_t>(kWarps, (size_t)smem_max / std::max<size_t>(ws_bytes, 1));
                    if (L.warps < 1) {
                        set_error("gpu eri: workspace of a quartet class exceeds shared memory");
                        return 10;
                    }
                    smem_need = std::max(smem_need, ws_bytes * L.warps);
                    L.t0 = all_tasks.size();
                    L.nt = v.size();
                    all_tasks.insert(all_tasks.end(), v.begin(), v.end());
                    voff_at.push_back(all_voff.size());
                    all_voff.insert(all_voff.end(), voff.begin(), voff.end());
                    launches.push_back(L);
                }
    if (launches.empty()) return 0;
    Task *dtasks = nullptr;
    int *dvoff = nullptr;
    constexpr int kStreams = 8;
    cudaStream_t st[kStreams] = {};
    auto fail = [&](const char *m) {
        for (cudaStream_t x : st)
            if (x) cudaStreamDestroy(x);
        cudaFree(dtasks); cudaFree(dvoff);
        set_error(std::string("gpu eri: ") + m);
        return 10;
    };
    const auto tk0 = std::chrono::steady_clock::now();
    if (cudaMalloc(&dtasks, all_tasks.size() * sizeof(Task)) != cudaSuccess) return fail("task allocation");
    if (cudaMalloc(&dvoff, all_voff.size() * sizeof(int)) != cudaSuccess) return fail("table allocation");
    if (cudaMemcpy(dtasks, all_tasks.data(), all_tasks.size() * sizeof(Task), cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(dvoff, all_voff.data(), all_voff.size() * sizeof(int), cudaMemcpyHostToDevice) != cudaSuccess)
        return fail("upload");
    if (cudaFuncSetAttribute(k_eri, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_need) != cudaSuccess)
        return fail("shared-memory attribute");
    for (cudaStream_t &x : st)
        if (cudaStreamCreateWithFlags(&x, cudaStreamNonBlocking) != cudaSuccess) return fail("stream");
    std::vector<size_t> ord(launches.size());
    for (size_t k = 0; k < ord.size(); k++) ord[k] = k;
    std::sort(ord.begin(), ord.end(), [&](size_t a, size_t b) {
        return (double)launches[a].nt * launches[a].C.T > (double)launches[b].nt * launches[b].C.T;
    });
    for (size_t k = 0; k < ord.size(); k++) {
        Launch &L = launches[ord[k]];
        L.C.voff = dvoff + voff_at[ord[k]];
        const size_t smem = (size_t)L.C.ws * sizeof(double) * L.warps;
        const long long nblk = std::min<long long>(((long long)L.nt + L.warps - 1) / L.warps, (long long)n_sm * 32);
        k_eri<<<(unsigned)nblk, 32 * L.warps, smem, st[k % kStreams]>>>(L.C, dtasks + L.t0, (int)L.nt, s->ssp, s->P,
                                                                        s->pe, s->K, s->ip, t->boys, dout);
        if (cudaGetLastError() != cudaSuccess) return fail("kernel launch");
    }
    for (cudaStream_t x : st)
        if (cudaStreamSynchronize(x) != cudaSuccess) return fail("kernel");
    for (cudaStream_t &x : st) {
        cudaStreamDestroy(x);
        x = nullptr;
    }
    cudaFree(dtasks);
    cudaFree(dvoff);
    *kms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - tk0).count();
    return 0;
}

static bool setup_verbose_env()
{
    const char *v = std::getenv("H2G_SETUP_VERBOSE");
    return v != nullptr && v[0] == '1';
}

static int eri_blocks_range(EriSet *s, Tables *t, EriReq *reqs, size_t n_req)
{
    auto nbfp = [&](int sp) { return ncart(s->host[sp].am1) * ncart(s->host[sp].am2); };
    std::vector<long long> boff(n_req + 1, 0);
    std::vector<BlockSpec> blocks(n_req);
    for (size_t r = 0; r < n_req; r++) {
        EriReq &q = reqs[r];
        int nr = 0, ncl = 0;
        for (int b : q.bra) nr += nbfp(b);
        for (int k : q.ket) ncl += nbfp(k);
        q.nrow = nr;
        q.ncol = ncl;
        boff[r + 1] = boff[r] + (long long)nr * ncl;
        blocks[r] = BlockSpec{q.bra.data(), q.ket.data(), (int)q.bra.size(), (int)q.ket.size(), q.sym, boff[r], ncl};
    }
    const long long total = boff.back();
    if (total == 0) return 0;
    double *dout = nullptr;
    if (cudaMalloc(&dout, (size_t)total * sizeof(double)) != cudaSuccess) {
        set_error("gpu eri: output allocation");
        return 10;
    }
    double kms = 0.0;
    int rc = launch_eri(s, t, blocks, dout, &kms);
    if (rc) {
        cudaFree(dout);
        return rc;
    }
    const auto tc0 = std::chrono::steady_clock::now();
    std::vector<double> host((size_t)total);
    rc = cudaMemcpy(host.data(), dout, (size_t)total * sizeof(double), cudaMemcpyDeviceToHost) == cudaSuccess ? 0 : 10;
    cudaFree(dout);
    if (rc) {
        set_error("gpu eri: copy back");
        return rc;
    }
    const auto tc1 = std::chrono::steady_clock::now();
    for (size_t r = 0; r < n_req; r++) {
        EriReq &q = reqs[r];
        for (int i = 0; i < q.nrow; i++)
            std::memcpy(q.out + (size_t)i * q.ld, host.data() + boff[r] + (size_t)i * q.ncol,
                        sizeof(double) * q.ncol);
    }
    const auto tc2 = std::chrono::steady_clock::now();
    if (setup_verbose_env())
        std::fprintf(stderr, "gpu eri: %zu blocks, %.1f M integrals: kernels %.1f ms, copy %.1f ms, scatter %.1f ms\n",
                     n_req, total / 1e6, kms, std::chrono::duration<double, std::milli>(tc1 - tc0).count(),
                     std::chrono::duration<double, std::milli>(tc2 - tc1).count());
    return 0;
}

/* ---- proxy-point potentials and sketches for the nested bases ---- */

namespace eri {

constexpr int kNaiL = 2 * kMaxAm;                                 /* la + lb  */
constexpr int kNaiV = 70;        /* compact [e]^(m), m <= L - |e|, for L = 4 */
constexpr int kNaiAcc = 31;      /* [e] for la <= |e| <= L (la = 2, L = 4)   */
constexpr int kNaiLvl = 48;      /* largest HRR level (la = lb = 2, j = 1)   */

/* One bra shell pair against a run of point charges: rows of the pair at
 * out_off (leading dimension ld), one column per point. */
struct NaiTask {
    int sp, npt;
    long long pt_off, out_off;
    int ld, pad_;
};

/* Potential integrals -<a| 1/|r - C| |b> of unit point charges: one thread
 * per point, the pair's primitive pairs in order. Obara-Saika recurrence
 * [e + 1_i]^(m) = PA_i [e]^(m) - PC_i [e]^(m+1) + e_i / (2p) ([e - 1_i]^(m)
 * - [e - 1_i]^(m+1)) from [0]^(m) = -2 pi / p K F_m(p |PC|^2), contraction,
 * then the horizontal recurrence to (a, b) - the host engine's
 * h2g_potential_points, point by point. */
__global__ void __launch_bounds__(128) k_nai(const NaiTask *__restrict__ tasks, const Ssp *__restrict__ ssp,
                                             const double *__restrict__ P, const double *__restrict__ pe,
                                             const double *__restrict__ K, const double *__restrict__ boys_tab,
                                             const double *__restrict__ px, const double *__restrict__ py,
                                             const double *__restrict__ pz, double *__restrict__ out)
{
    const NaiTask tk = tasks[blockIdx.x];
    const Ssp pr = ssp[tk.sp];
    const int la = pr.am1, lb = pr.am2, L = la + lb;
    const int ne = c_cum[L + 1], e0 = c_cum[la];
    const int na = ncart(la), nb = ncart(lb);
    /* compact offsets of [e]^(m): components of total l hold L - l + 1 orders */
    int loff[kNaiL + 2];
    loff[0] = 0;
    for (int l = 0; l <= L; l++) loff[l + 1] = loff[l] + ncart(l) * (L - l + 1);
    const double AB[3] = {pr.A[0] - pr.B[0], pr.A[1] - pr.B[1], pr.A[2] - pr.B[2]};
    for (int pt = threadIdx.x; pt < tk.npt; pt += blockDim.x) {
        const double C[3] = {px[tk.pt_off + pt], py[tk.pt_off + pt], pz[tk.pt_off + pt]};
        double acc[kNaiAcc];
        for (int e = 0; e < ne - e0; e++) acc[e] = 0.0;
        double V[kNaiV];
        for (int k = 0; k < pr.nprim; k++) {
            const int pi = pr.poff + k;
            const double p = pe[pi];
            double PA[3], PC[3], PC2 = 0.0;
#pragma unroll
            for (int d = 0; d < 3; d++) {
                const double Pd = P[3 * pi + d];
                PA[d] = Pd - pr.A[d];
                PC[d] = Pd - C[d];
                PC2 += PC[d] * PC[d];
            }
            double F[kNaiL + 1];
            boys(L, p * PC2, boys_tab, F);
            const double pref = -1.0 * 2.0 * M_PI / p * K[pi];
            for (int m = 0; m <= L; m++) V[m] = pref * F[m];
            const double i2p = 0.5 / p;
            for (int c = 1; c < ne; c++) {
                const int lc = lsum(c), d = c_dir[c], e = c_prev[c], e2 = c_prev2[c];
                const int le = lc - 1;
                const double ei = (double)(c_lxyz[c][d] - 1);
                double *vc = V + loff[lc] + (c - c_cum[lc]) * (L - lc + 1);
                const double *ve = V + loff[le] + (e - c_cum[le]) * (L - le + 1);
                if (e2 >= 0) {
                    const int le2 = lc - 2;
                    const double *ve2 = V + loff[le2] + (e2 - c_cum[le2]) * (L - le2 + 1);
                    for (int m = 0; m <= L - lc; m++)
                        vc[m] = PA[d] * ve[m] - PC[d] * ve[m + 1] + ei * i2p * (ve2[m] - ve2[m + 1]);
                } else {
                    for (int m = 0; m <= L - lc; m++) vc[m] = PA[d] * ve[m] - PC[d] * ve[m + 1];
                }
            }
            for (int e = e0; e < ne; e++) {
                const int le = lsum(e);
                acc[e - e0] += V[loff[le] + (e - c_cum[le]) * (L - le + 1)];
            }
        }
        /* horizontal recurrence (a, b + 1_i) = (a + 1_i, b) + AB_i (a, b) */
        double b0[kNaiLvl], b1[kNaiLvl];
        const double *cur = acc;
        int nbp = 1;
        for (int j = 1; j <= lb; j++) {
            const int nbj = ncart(j), emax = c_cum[L - j + 1];
            double *nxt = (j & 1) ? b0 : b1;
            for (int e = e0; e < emax; e++)
                for (int ib = 0; ib < nbj; ib++) {
                    const int bf = c_cum[j] + ib, d = c_dir[bf], bp = c_prev[bf] - c_cum[j - 1];
                    const int ep = c_plus[e][d];
                    nxt[(e - e0) * nbj + ib] = cur[(ep - e0) * nbp + bp] + AB[d] * cur[(e - e0) * nbp + bp];
                }
            cur = nxt;
            nbp = nbj;
        }
        for (int ab = 0; ab < na * nb; ab++) out[tk.out_off + (long long)ab * tk.ld + pt] = cur[ab];
    }
}

/* Columns of a sparse sign sketch: Y[i][j] = sum_l val[j][l] X[i][col[j][l]]
 * for i < nrow, j < n (the host sketch_apply, same order of sums). */
struct SkJob {
    long long x_off, s_off, y_off;
    int ldx, nrow, nnz, n, ldy, pad_;
};

__global__ void __launch_bounds__(256) k_sketch(const SkJob *__restrict__ jobs, const double *__restrict__ X,
                                                const int *__restrict__ scol, const double *__restrict__ sval,
                                                double *__restrict__ Y)
{
    const SkJob jb = jobs[blockIdx.y];
    const long long total = (long long)jb.nrow * jb.n;
    for (long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
         idx += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(idx / jb.n), j = (int)(idx - (long long)i * jb.n);
        const double *xi = X + jb.x_off + (long long)i * jb.ldx;
        const int *c = scol + jb.s_off + (long long)j * jb.nnz;
        const double *v = sval + jb.s_off + (long long)j * jb.nnz;
        double r = 0.0;
        for (int l = 0; l < jb.nnz; l++) r += v[l] * xi[c[l]];
        Y[jb.y_off + (long long)i * jb.ldy + j] = r;
    }
}

}  // namespace eri

static int u_blocks_range(EriSet *s, Tables *t, UReq *reqs, size_t n_req);

int gpu_u_blocks(EriSet *s, std::vector<UReq> &reqs)
{
    if (cudaSetDevice(s->device) != cudaSuccess) {
        set_error("gpu eri: cannot select the device of the shell pairs");
        return 10;
    }
    Tables *t;
    int rc = ensure_tables(&t);
    if (rc) return rc;
    auto nbfp = [&](int sp) { return ncart(s->host[sp].am1) * ncart(s->host[sp].am2); };
    for (UReq &q : reqs) {
        q.nrow = 0;
        for (int i = 0; i < q.nbra; i++) {
            if (q.bra[i] < 0 || q.bra[i] >= s->n_sp) { set_error("gpu eri: shell pair out of range"); return 3; }
            q.nrow += nbfp(q.bra[i]);
        }
        q.ncol_ff = 0;
        for (int i = 0; i < q.nket; i++) {
            if (q.ket[i] < 0 || q.ket[i] >= s->n_sp) { set_error("gpu eri: shell pair out of range"); return 3; }
            q.ncol_ff += nbfp(q.ket[i]);
        }
        /* every sketch index must address a column of its block */
        for (long long k = 0; k < (long long)q.nrow * q.s1_nnz; k++)
            if (q.s1_col[k] < 0 || q.s1_col[k] >= q.npt) { set_error("gpu eri: sketch column out of range"); return 3; }
        for (long long k = 0; k < (long long)q.nrow * q.s2_nnz; k++)
            if (q.s2_col[k] < 0 || q.s2_col[k] >= q.ncol_ff) { set_error("gpu eri: sketch column out of range"); return 3; }
    }
    /* requests in groups of at most 2^27 doubles of unsketched blocks */
    size_t i = 0;
    while (i < reqs.size()) {
        size_t j = i;
        long long tot = 0;
        while (j < reqs.size()) {
            const long long n = (long long)reqs[j].nrow * (reqs[j].npt + reqs[j].ncol_ff);
            if (j > i && tot + n > (1LL << 27)) break;
            tot += n;
            j++;
        }
        rc = u_blocks_range(s, t, reqs.data() + i, j - i);
        if (rc) return rc;
        i = j;
    }
    return 0;
}

static int u_blocks_range(EriSet *s, Tables *t, UReq *reqs, size_t n_req)
{
    auto nbfp = [&](int sp) { return ncart(s->host[sp].am1) * ncart(s->host[sp].am2); };
    /* device layout: X = [potential block | ERI block] per request, A =
     * nrow x 2 nrow per request, points and sketches concatenated */
    std::vector<long long> xn(n_req), xe(n_req), ao(n_req + 1, 0), po(n_req), s1o(n_req), s2o(n_req);
    long long nx = 0, np = 0, ns = 0;
    std::vector<BlockSpec> blocks;
    std::vector<NaiTask> nai;
    std::vector<SkJob> jobs;
    for (size_t r = 0; r < n_req; r++) {
        const UReq &q = reqs[r];
        xn[r] = nx;
        nx += (long long)q.nrow * q.npt;
        xe[r] = nx;
        nx += (long long)q.nrow * q.ncol_ff;
        ao[r + 1] = ao[r] + 2LL * q.nrow * q.nrow;
        po[r] = np;
        np += q.npt;
        s1o[r] = ns;
        ns += (long long)q.nrow * q.s1_nnz;
        s2o[r] = ns;
        ns += (long long)q.nrow * q.s2_nnz;
        if (q.nrow == 0) continue;
        if (q.nket > 0) blocks.push_back(BlockSpec{q.bra, q.ket, q.nbra, q.nket, false, xe[r], q.ncol_ff});
        int row = 0;
        for (int b = 0; b < q.nbra; b++) {
            if (q.npt > 0) nai.push_back(NaiTask{q.bra[b], q.npt, po[r], xn[r] + (long long)row * q.npt, q.npt, 0});
            row += nbfp(q.bra[b]);
        }
        jobs.push_back(SkJob{xn[r], s1o[r], ao[r], q.npt, q.nrow, q.s1_nnz, q.nrow, 2 * q.nrow, 0});
        jobs.push_back(SkJob{xe[r], s2o[r], ao[r] + q.nrow, q.ncol_ff, q.nrow, q.s2_nnz, q.nrow, 2 * q.nrow, 0});
    }
    if (ao[n_req] == 0) return 0;
    std::vector<double> pts(3 * (size_t)std::max<long long>(np, 1)), sval((size_t)std::max<long long>(ns, 1));
    std::vector<int> scol((size_t)std::max<long long>(ns, 1));
    for (size_t r = 0; r < n_req; r++) {
        const UReq &q = reqs[r];
        if (q.npt > 0) {
            std::memcpy(pts.data() + po[r], q.px, sizeof(double) * q.npt);
            std::memcpy(pts.data() + np + po[r], q.py, sizeof(double) * q.npt);
            std::memcpy(pts.data() + 2 * np + po[r], q.pz, sizeof(double) * q.npt);
        }
        const size_t n1 = (size_t)q.nrow * q.s1_nnz, n2 = (size_t)q.nrow * q.s2_nnz;
        if (n1 > 0) {
            std::memcpy(scol.data() + s1o[r], q.s1_col, sizeof(int) * n1);
            std::memcpy(sval.data() + s1o[r], q.s1_val, sizeof(double) * n1);
        }
        if (n2 > 0) {
            std::memcpy(scol.data() + s2o[r], q.s2_col, sizeof(int) * n2);
            std::memcpy(sval.data() + s2o[r], q.s2_val, sizeof(double) * n2);
        }
    }
    double *dX = nullptr, *dA = nullptr, *dpts = nullptr, *dsval = nullptr;
    int *dscol = nullptr;
    NaiTask *dnai = nullptr;
    SkJob *djobs = nullptr;
    auto release = [&]() {
        cudaFree(dX); cudaFree(dA); cudaFree(dpts); cudaFree(dsval); cudaFree(dscol); cudaFree(dnai); cudaFree(djobs);
    };
    auto fail = [&](const char *m) {
        release();
        set_error(std::string("gpu eri (nested bases): ") + m);
        return 10;
    };
    const auto t0 = std::chrono::steady_clock::now();
    if (cudaMalloc(&dX, (size_t)std::max<long long>(nx, 1) * sizeof(double)) != cudaSuccess ||
        cudaMalloc(&dA, (size_t)ao[n_req] * sizeof(double)) != cudaSuccess ||
        cudaMalloc(&dpts, pts.size() * sizeof(double)) != cudaSuccess ||
        cudaMalloc(&dsval, sval.size() * sizeof(double)) != cudaSuccess ||
        cudaMalloc(&dscol, scol.size() * sizeof(int)) != cudaSuccess ||
        cudaMalloc(&dnai, std::max<size_t>(nai.size(), 1) * sizeof(NaiTask)) != cudaSuccess ||
        cudaMalloc(&djobs, std::max<size_t>(jobs.size(), 1) * sizeof(SkJob)) != cudaSuccess)
        return fail("allocation");
    if (cudaMemcpy(dpts, pts.data(), pts.size() * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(dsval, sval.data(), sval.size() * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(dscol, scol.data(), scol.size() * sizeof(int), cudaMemcpyHostToDevice) != cudaSuccess ||
        (!nai.empty() && cudaMemcpy(dnai, nai.data(), nai.size() * sizeof(NaiTask), cudaMemcpyHostToDevice) != cudaSuccess) ||
        (!jobs.empty() && cudaMemcpy(djobs, jobs.data(), jobs.size() * sizeof(SkJob), cudaMemcpyHostToDevice) != cudaSuccess))
        return fail("upload");
    /* potentials on a stream of their own while the ERI classes run on
     * theirs; the sketches after both */
    cudaStream_t sn = nullptr;
    if (cudaStreamCreateWithFlags(&sn, cudaStreamNonBlocking) != cudaSuccess) return fail("stream");
    auto fail_s = [&](const char *m) {
        cudaStreamSynchronize(sn);
        cudaStreamDestroy(sn);
        return fail(m);
    };
    if (!nai.empty()) {
        k_nai<<<(unsigned)nai.size(), 128, 0, sn>>>(dnai, s->ssp, s->P, s->pe, s->K, t->boys, dpts, dpts + np,
                                                    dpts + 2 * np, dX);
        if (cudaGetLastError() != cudaSuccess) return fail_s("potential kernel launch");
    }
    double kms = 0.0;
    if (!blocks.empty()) {
        const int rc = launch_eri(s, t, blocks, dX, &kms);
        if (rc) {
            cudaStreamSynchronize(sn);
            cudaStreamDestroy(sn);
            release();
            return rc;
        }
    }
    for (size_t j0 = 0; j0 < jobs.size(); j0 += 65535) {   /* grid.y is at most 65535 */
        dim3 grid(64, (unsigned)std::min<size_t>(65535, jobs.size() - j0));
        k_sketch<<<grid, 256, 0, sn>>>(djobs + j0, dX, dscol, dsval, dA);
        if (cudaGetLastError() != cudaSuccess) return fail_s("sketch kernel launch");
    }
    if (cudaStreamSynchronize(sn) != cudaSuccess) return fail_s("kernels");
    cudaStreamDestroy(sn);
    const auto t1 = std::chrono::steady_clock::now();
    std::vector<double> host((size_t)ao[n_req]);
    if (cudaMemcpy(host.data(), dA, host.size() * sizeof(double), cudaMemcpyDeviceToHost) != cudaSuccess)
        return fail("copy back");
    release();
    for (size_t r = 0; r < n_req; r++) {
        UReq &q = reqs[r];
        const int w = 2 * q.nrow;
        for (int i = 0; i < q.nrow; i++)
            std::memcpy(q.out + (size_t)i * q.ld, host.data() + ao[r] + (size_t)i * w, sizeof(double) * w);
    }
    if (setup_verbose_env())
        std::fprintf(stderr, "gpu nested-basis blocks: %zu nodes, %.1f M potentials + ERIs, %zu potential rows: "
                     "kernels %.1f ms (ERI classes %.1f ms), copy back and scatter %.1f ms\n", n_req, nx / 1e6,
                     nai.size(), std::chrono::duration<double, std::milli>(t1 - t0).count(), kms,
                     std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t1).count());
    return 0;
}

}  // namespace h2g
