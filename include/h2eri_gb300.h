/*
 * h2eri_gb300: GPU (sm_103a) drop-in for the H2P-ERI C API.
 *
 * The entry points in the first block keep the reference names, argument
 * meanings and void/abort error behaviour; each comment names the reference
 * declaration it replaces. Set-up (init, shells, partition, build_H2) runs on
 * the host once per geometry; the hot path (matvec, Coulomb, exchange) runs on
 * the GPU with the H2 blocks resident in device memory after the first call
 * (or an explicit H2ERI_gpu_upload). There is no CPU fallback: on a machine
 * without a usable CUDA device the hot-path calls print the reason and abort,
 * the int-returning extensions return a nonzero status instead.
 *
 * Not re-entrant per H2ERI_p (same as the reference): one host thread at a
 * time may use a given structure.
 */
#ifndef H2ERI_GB300_H
#define H2ERI_GB300_H

#include "h2eri_types.h"

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------------ */
/* Reference API                                                             */
/* ------------------------------------------------------------------------ */

/* replaces H2P-ERI src/H2ERI_typedef.h:169 */
void H2ERI_init(H2ERI_p *h2eri_, const double scr_tol, const double ext_tol, const double QR_tol);
/* replaces src/H2ERI_typedef.h:174; also releases the GPU state */
void H2ERI_destroy(H2ERI_p h2eri);
/* replaces src/H2ERI_typedef.h:179; adds GPU columns when timings exist */
void H2ERI_print_statistic(H2ERI_p h2eri);
/* replaces src/CMS.h:49 */
void CMS_read_mol_file(const char *mol_fname, int *natom_, int *nshell_, shell_t **shells_);
/* replaces src/CMS.h:55 */
void CMS_destroy_shells(const int nshell, shell_t *shells);
/* replaces src/H2ERI_shell_operations.h:25 */
void H2ERI_process_shells(H2ERI_p h2eri);
/* replaces src/H2ERI_partition.h:28 */
void H2ERI_partition(H2ERI_p h2eri);
/* replaces src/H2ERI_build_H2.h:16; only BD_JIT == 0 is supported (the GPU
 * path needs the blocks built ahead of time); BD_JIT == 1 aborts */
void H2ERI_build_H2(H2ERI_p h2eri, const int BD_JIT);
/* replaces src/H2ERI_matvec.h:16: y = A x over the krnl_mat_size SSP
 * basis-function-pair space; x, y host arrays */
void H2ERI_matvec(H2ERI_p h2eri, const double *x, double *y);
/* replaces src/H2ERI_build_Coulomb.h:16: J from a symmetric density, both
 * num_bf x num_bf row-major host arrays */
void H2ERI_build_Coulomb(H2ERI_p h2eri, const double *den_mat, double *J_mat);
/* replaces src/H2ERI_build_exchange.h:16: K from a symmetric density */
void H2ERI_build_exchange(H2ERI_p h2eri, const double *den_mat, double *K_mat);
/* replace src/H2ERI_build_exchange.h:19,22; the GPU exchange keeps its own
 * device workspace, these only manage the host-side field */
void H2ERI_exchange_workbuf_init(H2ERI_p h2eri);
void H2ERI_exchange_workbuf_free(H2ERI_p h2eri);
/* replaces src/H2ERI_typedef.c:303 (exported, undeclared in the reference) */
void H2E_reset_timers(H2ERI_p h2eri);

/* ------------------------------------------------------------------------ */
/* GPU extensions (no counterpart in the reference)                          */
/* ------------------------------------------------------------------------ */

/* Precision of the far-field (U, B) blocks on the GPU. */
#define H2ERI_GPU_FP64   0   /* everything FP64                                   */
#define H2ERI_GPU_MIXED  1   /* U and leaf self-interaction D blocks as FP32 hi+lo */
                             /* pairs, other B and D blocks as FP32; products    */
                             /* accumulated in FP32 to ~2^-44, sums in FP64;     */
                             /* J relative error ~5e-9 at QR tolerance 1e-8      */

/* Upload the H2 blocks and tree arrays of a built structure to the current
 * CUDA device. Called implicitly by the first hot-path call. Returns 0 on
 * success. */
int H2ERI_gpu_upload(H2ERI_p h2eri);
/* Free the device copy of a structure (called by H2ERI_destroy). */
void H2ERI_gpu_release(H2ERI_p h2eri);
/* Select the far-field precision for subsequent calls (default FP64).
 * Re-uploads the far-field blocks if needed. Returns 0 on success. */
int H2ERI_gpu_set_precision(H2ERI_p h2eri, int mode);
/* Device memory (no counterpart in the reference): a structure in the mixed
 * mode reads only its FP32 / float-pair copy and the tensor-core slices, so
 * its FP64 copy (about 40 % of its device footprint) can be freed, e.g. to
 * keep a large batch of molecules resident in HBM. Afterwards the structure
 * refuses H2ERI_gpu_set_precision(.., FP64) with an error; H2ERI_gpu_release
 * and a new upload bring the FP64 mode back. Returns 0, or 3 when the
 * structure is not in the mixed mode. */
int H2ERI_gpu_drop_fp64(H2ERI_p h2eri);
/* Message of the last failure of any gpu extension call on this thread
 * ("" if none). */
const char *H2ERI_gpu_last_error(void);
/* Self-test of the kernels' bounded waits: launches one CTA that waits on an
 * mbarrier nothing arrives at, with a limit of `cycles` SM clock cycles, the
 * way the tile kernels wait for their TMA copies. Returns 1 when the wait
 * gave up and the error word reported it, 0 when it did not, negative on a
 * CUDA error. The device stays usable afterwards. */
int H2ERI_gpu_selftest_wait_timeout(long long cycles);

/* The same wait enqueued on a stream (void* cudaStream_t, NULL = the
 * structure's own), recording its expiry in the structure's error word the
 * way the kernels of the asynchronous entry points do; returns after
 * enqueueing (0) and leaves the report to H2ERI_gpu_check. */
int H2ERI_gpu_selftest_wait_timeout_async(H2ERI_p h2eri, long long cycles, void *stream);
/* Failure-detection check of the persistent mixed-mode kernel (mixed
 * precision only): one matvec of a zero vector with the item count of the
 * first range raised by one, so the range after it waits for an item that
 * never completes; that wait gives up after `cycles` SM cycles, the kernel
 * returns, and the expiry must be reported. The count is restored. Returns
 * 1 when the expiry was reported, 0 when not, > 1 on error. */
int H2ERI_gpu_selftest_persist_timeout(H2ERI_p h2eri, long long cycles);
/* After asynchronous calls (the _device variants and
 * H2ERI_matvec_device_noalloc return before their kernels run): waits for
 * the structure's own streams and returns 11, with a message in
 * H2ERI_gpu_last_error, if any of its kernels gave up a bounded wait (or
 * found its shared memory misaligned and did nothing) since the last check;
 * 0 otherwise. The record is cleared. Synchronise the stream passed to the
 * asynchronous calls first. The host-array calls check by themselves. */
int H2ERI_gpu_check(H2ERI_p h2eri);

/* y = A x for nvec vectors stored back to back ([nvec][krnl_mat_size]),
 * host arrays. Returns 0 on success. */
int H2ERI_matvec_multi(H2ERI_p h2eri, int nvec, const double *x, double *y);
/* Same on device arrays, enqueued on a CUDA stream (cudaStream_t passed as
 * void*, NULL = the library's stream); returns after enqueueing. */
int H2ERI_matvec_device(H2ERI_p h2eri, int nvec, const double *d_x, double *d_y, void *stream);
/* J for n_den densities stored back to back ([n_den][num_bf][num_bf]) on the
 * host. Returns 0 on success. */
int H2ERI_build_Coulomb_multi(H2ERI_p h2eri, int n_den, const double *den_mats, double *J_mats);
/* Same on device arrays, enqueued on a stream. */
int H2ERI_build_Coulomb_device(H2ERI_p h2eri, int n_den, const double *d_den, double *d_J, void *stream);
/* J for n structures (molecules of any size) in one call, device arrays:
 * d_dens[i] / d_Js[i] hold n_den[i] densities / J matrices of h2eris[i]
 * ([n_den][num_bf][num_bf]). The builds are forked from `stream` onto each
 * structure's own streams, run concurrently and are joined back to `stream`.
 * A structure may appear once per call. No counterpart in the reference
 * (its callers loop over H2ERI_build_Coulomb). Returns 0 on success. */
int H2ERI_build_Coulomb_batch(int n, H2ERI_p *h2eris, const int *n_den, const double *const *d_dens,
                              double *const *d_Js, void *stream);
/* K for n_den densities stored back to back ([n_den][num_bf][num_bf]) on the
 * host, one after the other. Returns 0 on success. */
int H2ERI_build_exchange_multi(H2ERI_p h2eri, int n_den, const double *den_mats, double *K_mats);
/* K on device arrays, enqueued on a stream. Returns 0 on success. */
int H2ERI_build_exchange_device(H2ERI_p h2eri, const double *d_den, double *d_K, void *stream);
/* Figures of the exchange plan: out[0] flops per K build, out[1] device time
 * of the last host-array K build (ms), out[2] number of n ranges the build is
 * split into, out[3] bytes of the G/H work tensors, out[4] near-field work
 * items, out[5] kernel launches per K build, out[6] 1 when the mixed mode's
 * products run on the tensor cores (bf16x3 splits, the default), 0 on the
 * FP32 SIMT kernel (H2G_K_TC=0 when the first mixed K build runs), -1 before
 * the first mixed K build. Returns the number of values written (<= n), or
 * < 0. */
int H2ERI_gpu_exchange_report(H2ERI_p h2eri, double *out, int n);
/* Cap the device memory of the exchange work tensors (bytes; 0 = 40 % of
 * the free memory, at most 16 GB). K is then built in more ranges of the
 * density's column index, with the same result. Returns 0 on success. */
int H2ERI_gpu_set_exchange_memory(H2ERI_p h2eri, double bytes);
/* Build the exchange plan on the host only (no device calls), sized as if
 * device_bytes of device memory were free, and check that every access of
 * every planned kernel stays inside its buffer. out[0] flops per K build,
 * out[1] number of n ranges, out[2] bytes of the work tensors, out[3]
 * near-field work items, out[4] GEMM tiles. Returns 0 if the plan is
 * consistent. */
int H2ERI_exchange_plan_check(H2ERI_p h2eri, double device_bytes, double *out, int n);

/* y = A x for one vector on device arrays, allocating no device memory.
 * No counterpart in the reference. For callers that must not allocate after
 * set-up (a fixed device-memory budget or a memory pool owned by the host
 * application, or loops where cudaMalloc/cudaFree would synchronise the
 * device). Requires the structure to be on the GPU already
 * (H2ERI_gpu_upload). The intermediates live in one fixed 16 MiB device
 * array shared by all calls; larger representations (2 * sum of ranks +
 * low-rank intermediates > 2^21 doubles, H2ERI_gpu_report out[13]) are
 * rejected with an error (status 4; H2G_NOALLOC_LIMIT=<doubles> in the
 * environment lowers the limit, never raises it). Null vectors are rejected
 * (status 3). Each call clears the array first; calls whose GPU work
 * overlaps race on it. The array's device address is looked up when the
 * structure is uploaded, so the call itself only reads it. Returns 0 after
 * enqueueing; H2ERI_gpu_check reports a kernel's expired wait afterwards. */
int H2ERI_matvec_device_noalloc(H2ERI_p h2eri, const double *d_x, double *d_y, void *stream);

/* Autotuner (no counterpart in the reference): runs every candidate launch
 * configuration of this structure at n_den densities per launch in its
 * current precision on the device, times each with CUDA events, and keeps
 * the fastest. Candidates: rows per tile of the single-density kernels
 * (0: chosen per range, the tallest of 512..64 that gives the range two
 * waves of CTAs; or 512, 256, 128 for all ranges); in the mixed mode the persistent launch (the whole
 * matvec in one launch) or one launch per range with tiles per CTA (2, 1)
 * and near-field lanes on their own streams or one; for several densities
 * in the mixed mode also the tensor-core kernel (n_SM or n_SM / 2 CTAs per
 * launch) against the single-density kernels. The choice is cached per structure shape,
 * precision and density-count class in the process and, with
 * H2G_TUNE_FILE=<path> in the environment, in that file, which later
 * processes read when a structure of the same shape is uploaded or changes
 * precision. Synchronises the device; takes about 0.1-1 s. out: [0] ms per
 * matvec with the choice, [1] ms before tuning, [2] candidates timed,
 * [3..8] the choice (tile rows, tiles per CTA, near-field lanes concurrent,
 * density count from which the tensor-core kernel runs, its CTA divisor,
 * persistent launch), [9..] ms of each candidate. Returns the number of
 * values written, or < 0. */
int H2ERI_gpu_autotune(H2ERI_p h2eri, int n_den, double *out, int n);

/* Set-up on the GPU (no counterpart in the reference): when a CUDA device is
 * present and H2G_SETUP_GPU is not 0, H2ERI_build_H2 evaluates the dense
 * near-field (D) and full coupling (B) blocks of electron-repulsion
 * integrals on the GPU (same recurrences and tables as the host engine;
 * shells up to d) and compresses them on the host as before. This check
 * evaluates up to max_blocks blocks of each kind (diagonal near-field,
 * inadmissible near-field, coupling) of a built structure with both
 * engines: out[0] largest |difference|, out[1] largest |value|, out[2]
 * elements compared, out[3] blocks compared, out[4] seconds on the GPU,
 * out[5] seconds on the host engine (one thread); out needs 6 values.
 * Returns 0, 9 without a usable device, or another error code. */
int H2ERI_gpu_setup_eri_check(H2ERI_p h2eri, int max_blocks, double *out);

/* Nested bases on the GPU (no counterpart in the reference): with a usable
 * device, H2ERI_build_H2 also evaluates the integrals of the nested-basis
 * construction on the GPU - the potentials of the proxy point charges
 * around each node and the ERIs with the overlapping far-field shell pairs,
 * each reduced by its sparse sign sketch on the device - and decomposes the
 * sketched matrices on the host (H2P-ERI src/H2ERI_build_H2.c:351-827
 * evaluates them on the host). This check evaluates the sketched matrices
 * of up to max_nodes nodes with both engines on the same inputs: out[0]
 * largest |difference|, out[1] largest |value|, out[2] elements compared,
 * out[3] nodes compared, out[4] seconds on the GPU, out[5] seconds on the
 * host engine (one thread); out needs 6 values. Returns 0, 9 without a
 * usable device, or another error code. */
int H2ERI_gpu_setup_u_check(H2ERI_p h2eri, int max_nodes, double *out);

/* Figures of the device copy, for reports. out[0] kernel launches per matvec
 * call (one vector block), out[1] algorithmic matrix bytes read per matvec,
 * out[2] algorithmic vector bytes per vector, out[3] flops per vector,
 * out[4..6] arena bytes of U, B, D, out[7..11] last timed phase durations
 * in ms (upward, coupling, downward, near field, total), out[12] far-field
 * precision mode, out[13] scratch doubles one matvec of one vector needs,
 * out[14..19] the launch choices in use (tile rows, tiles per CTA,
 * near-field lanes concurrent, density count from which the tensor-core
 * kernel runs, its CTA divisor, persistent launch; see H2ERI_gpu_autotune),
 * out[20..22] the persistent kernel's work list (items, CTAs, makespan in ms
 * of its host schedule simulation; 0 before its first use). In the mixed
 * single-density path with the persistent launch, the phase durations
 * out[7..9] all hold the whole launch. Returns the number of values written
 * (<= n), or < 0. */
int H2ERI_gpu_report(H2ERI_p h2eri, double *out, int n);

/* Save / load the H2 representation (tree, pair lists, U, B, D and the
 * basis-function bookkeeping used by J and K) in a self-describing binary
 * file, so the same blocks can be applied on another machine or process. */
int H2ERI_save_representation(H2ERI_p h2eri, const char *path);
int H2ERI_load_representation(const char *path, H2ERI_p *h2eri_);

#ifdef __cplusplus
}
#endif

#endif
