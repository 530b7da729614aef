/* GPU exchange (K) build: placeholder until the batched kernels land. */
#include "h2eri_gb300.h"
#include "h2g_gpu_api.h"
#include <cstdio>
#include <cstdlib>

namespace h2g {
void free_exchange_state(DevRep *d) { (void)d; }
}  // namespace h2g

extern "C" int H2ERI_build_exchange_device(H2ERI_p h2eri, const double *d_den, double *d_K, void *stream)
{
    (void)h2eri; (void)d_den; (void)d_K; (void)stream;
    h2g::set_error("H2ERI_build_exchange_device: not available in this build");
    return 20;
}

extern "C" void H2ERI_build_exchange(H2ERI_p h2eri, const double *den_mat, double *K_mat)
{
    (void)h2eri; (void)den_mat; (void)K_mat;
    std::fprintf(stderr, "[h2eri_gb300 FATAL] H2ERI_build_exchange: not available in this build\n");
    std::abort();
}
