/* Host set-up driver for the sanitizer test (tests/test_sanitize_setup_cpu.py):
 * the reference call sequence up to H2ERI_build_H2 and a save/load round
 * trip, built from the host sources alone with AddressSanitizer and
 * UndefinedBehaviorSanitizer. The GPU-side hooks the host code calls are
 * stubbed (nothing is uploaded here, and the set-up's integral blocks stay on
 * the host engine). */
#include <cstdio>
#include <cstdlib>

#include "h2eri_gb300.h"
#include "h2g_eri.h"

extern "C" void H2ERI_gpu_release(H2ERI_p) {}
extern "C" void h2g_gpu_print_statistic(H2ERI_p) {}
extern "C" const char *H2ERI_gpu_last_error(void) { return "the GPU hooks are stubbed in this test program"; }
namespace h2g {
int gpu_eri_usable() { return 0; }
int gpu_eri_create(int, const h2g_pair *const *, EriSet **out) { *out = nullptr; return 1; }
int gpu_eri_blocks(EriSet *, std::vector<EriReq> &) { return 1; }
int gpu_u_blocks(EriSet *, std::vector<UReq> &) { return 1; }
void gpu_eri_free(EriSet *) {}
}  // namespace h2g

int main(int argc, char **argv)
{
    if (argc < 4) return 2;
    H2ERI_p h;
    H2ERI_init(&h, 1e-10, 1e-10, std::atof(argv[2]));
    CMS_read_mol_file(argv[1], &h->natom, &h->nshell, &h->shells);
    H2ERI_process_shells(h);
    H2ERI_partition(h);
    H2ERI_build_H2(h, 0);
    if (H2ERI_save_representation(h, argv[3]) != 0) return 3;
    H2ERI_p g = nullptr;
    if (H2ERI_load_representation(argv[3], &g) != 0) return 4;
    std::printf("num_bf %d krnl %d n_node %d\n", h->num_bf, h->krnl_mat_size, h->n_node);
    H2ERI_destroy(g);
    H2ERI_destroy(h);
    return 0;
}
