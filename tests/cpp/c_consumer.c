/* A plain C99 consumer of the C ABI: compiles against include/ipic3d_gpu.h,
 * links the library, fills the default configuration and, without an sm_103
 * GPU, gets IPIC3D_E_NODEVICE from ipic3d_gpu_create with a message. */
#include <stdio.h>

#include "ipic3d_gpu.h"

int main(void) {
    ipic3d_config cfg;
    ipic3d_props props = {{2, 2, 2}, {1.0, 1.0, 1.0}, 0.1, 1.0, 0.0, {0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    ipic3d_ctx* ctx = NULL;
    char msg[256];
    int rc;
    ipic3d_gpu_config_default(&cfg);
    printf("defaults %d %d %d %d\n", cfg.precision, cfg.mover, cfg.solver, cfg.projector);
    rc = ipic3d_gpu_create(&props, &cfg, &ctx);
    ipic3d_gpu_last_error(msg, sizeof msg);
    printf("create %d %s\n", rc, rc ? msg : "");
    if (ctx) ipic3d_gpu_destroy(ctx);
    return 0;
}
