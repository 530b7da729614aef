/* Internal: GPU-side report hooks used by the host statistics printer. */
#ifndef H2G_GPU_STATS_H
#define H2G_GPU_STATS_H

#include "h2eri_types.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Prints device-arena sizes and the last device phase times, if any. */
void h2g_gpu_print_statistic(H2ERI_p h2eri);

#ifdef __cplusplus
}
#endif

#endif
