/* A plain C99 caller of the engine's C ABI: includes the public header and
 * calls the entry points that run on the host only (options, Holberg
 * coefficients, checkpoint schedule, filter weights, error strings), so it
 * runs without a GPU.  Prints one line per check; exits non-zero on the
 * first failure. */
#include <math.h>
#include <stdio.h>
#include <string.h>

#include "fwi_psv.h"

#define CHECK(c)                                           \
    do {                                                   \
        if (!(c)) {                                        \
            printf("FAIL %s:%d %s\n", __FILE__, __LINE__, #c); \
            return 1;                                      \
        }                                                  \
    } while (0)

int main(void)
{
    psv_options o;
    double hc[7], k[25];
    int acts[3 * 64], n = 0;
    long long adv = -1;

    psv_options_default(&o);
    CHECK(o.precision == 32 && o.storage == PSV_STORE_AUTO && o.use_graphs == 1);
    CHECK(o.hbm_budget_gb == 180.0 && o.chains == 0 && o.checkpoint_slots == 0);

    memset(hc, 0, sizeof(hc));
    CHECK(psv_holbergcoeff(4, 1, hc) == PSV_OK);
    CHECK(hc[1] > 1.0 && hc[2] < 0.0); /* 4th-order staggered weights */

    CHECK(psv_checkpoint_schedule(10, 3, acts, 64, &n, &adv) == PSV_OK);
    CHECK(n > 10 && adv == 8);       /* Griewank: 15 advances, 7 on the forward pass */
    CHECK(psv_checkpoint_schedule(10, 3, acts, 4, &n, &adv) == PSV_ERR_ARG);

    CHECK(psv_gauss_filter_kernel(2, k) == PSV_OK);
    {
        double s = 0.0;
        int i;
        for (i = 0; i < 25; i++) s += k[i];
        CHECK(fabs(s - 1.0) < 1e-14 && k[12] > k[0]);
    }
    CHECK(psv_gauss_filter_kernel(1, k) == PSV_ERR_ARG);
    CHECK(strlen(psv_last_error()) > 0);
    CHECK(strlen(psv_error_string(PSV_ERR_CUDA)) > 0);
    {
        /* a grid taller than a CUDA grid dimension is refused before any
         * device work, with or without a GPU */
        psv_grid g;
        psv_shots s;
        psv_plan *plan = NULL;
        memset(&g, 0, sizeof g);
        memset(&s, 0, sizeof s);
        g.nt = 1;
        g.nz = PSV_MAX_NZ + 1;
        g.nx = 8;
        CHECK(psv_plan_create(&g, &s, NULL, &plan) == PSV_ERR_UNSUPPORTED && plan == NULL);
        CHECK(PSV_MAX_SHOT_ELEMS == 2147483647LL && PSV_MAX_SHOTS == 65535);
    }
    printf("ok %d actions, device %d\n", n, psv_device_available());
    return 0;
}
