/* Mixed-precision far field: placeholder until the FP32 arenas land. */
#include "h2eri_gb300.h"
#include "h2g_gpu_api.h"

namespace h2g {
int set_precision_mode(DevRep *d, H2ERI_p h, int mode)
{
    (void)h;
    if (mode == H2ERI_GPU_FP64) { d->precision = 0; return 0; }
    set_error("mixed precision not available in this build");
    return 21;
}
}  // namespace h2g
