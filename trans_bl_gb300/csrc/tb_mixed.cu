// tb_mixed.cu -- mixed-precision form of the v-Poisson solve (placeholder
// until the FP32 multigrid lands; selecting it is rejected at set-up).
#include "tb_internal.h"

int tb_mixed_setup(tb_ctx* c) {
    (void)c;
    tb_set_error("mixed-precision form not available in this build");
    return TB_ERR_ARG;
}
void tb_mixed_free(tb_ctx* c) { (void)c; }
int tb_poi_uy_mixed(tb_ctx* c, const cplx* dwzdx, double erro) {
    (void)c; (void)dwzdx; (void)erro;
    tb_set_error("mixed-precision form not available in this build");
    return TB_ERR_ARG;
}
