/* A C program written against include/libcaps.h the way the reference's callers use the
 * API (src/caps_logdetD.c:176-215, examples/AuAl.c): caps_init, the setters, a Drude
 * callback through caps_set_epsilonm1 with caller-owned userdata, caps_logdetD,
 * caps_logdetD0, caps_mie, caps_free.  Linked against libcaps_gb300.so; it prints one
 * "name value" line per result, which tests/test_c_caller.py compares with the reference's
 * values. */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>

#include "libcaps.h"

int main(void)
{
    caps_t *bad = caps_init(-1.0, 1.0); /* L <= 0 or R <= 0: NULL (libcaps.c:186-187) */
    printf("init_invalid_is_null %d\n", bad == NULL);

    /* perfect reflectors, R/L = 20, ldim 140 */
    caps_t *caps = caps_init(20e-6, 1e-6);
    printf("set_ldim_zero %d\n", caps_set_ldim(caps, 0));
    printf("set_ldim %d\n", caps_set_ldim(caps, 140));
    printf("get_ldim %d\n", caps_get_ldim(caps));
    printf("set_epsrel_negative %d\n", caps_set_epsrel(caps, -1.0));
    printf("default_detalg_is_hodlr %d\n", caps_get_detalg(caps) == DETALG_HODLR);
    printf("pr_hodlr_xi1_m20 %.17g\n", caps_logdetD(caps, 1.0, 20));
    caps_set_detalg(caps, DETALG_LU);
    printf("pr_lu_xi1_m0 %.17g\n", caps_logdetD(caps, 1.0, 0));
    printf("pr_lu_xi1_m5 %.17g\n", caps_logdetD(caps, 1.0, 5));
    caps_free(caps);

    /* Drude metal through the callback (omega_p = 9 eV, gamma = 0.035 eV, in rad/s) */
    double userdata[2] = {9.0 / CAPS_hbar_eV, 0.035 / CAPS_hbar_eV};
    caps = caps_init(20e-6, 1e-6);
    caps_set_ldim(caps, 140);
    caps_set_detalg(caps, DETALG_LU);
    caps_set_epsilonm1(caps, caps_epsilonm1_drude, userdata);
    printf("drude_lu_xi3_m2 %.17g\n", caps_logdetD(caps, 3.0, 2));
    printf("drude_lu_xi12_m7 %.17g\n", caps_logdetD(caps, 12.0, 7));
    caps_free(caps);

    /* Mie coefficients of a Drude sphere (src/tests/test_mie_drude.c: R = L = 100 um,
     * omega_p = 5e4 c/(L+R), gamma = c/(L+R), xi = 1e-4, l = 1) */
    {
        const double R = 1e-4, L = 1e-4;
        double ud[2] = {5e4 * CAPS_c / (L + R), 1.0 * CAPS_c / (L + R)};
        double lna, lnb;
        caps_t *s = caps_init(R, L);
        caps_set_epsilonm1(s, caps_epsilonm1_drude, ud);
        caps_mie(s, 1e-4, 1, &lna, &lnb);
        printf("mie_drude_lna %.17g\n", lna);
        printf("mie_drude_lnb %.17g\n", lnb);
        caps_free(s);
    }

    /* xi = 0, perfect reflectors, R/L = 1000, ldim 12000, m = 0 (src/tests/test_logdetD.c:128-142) */
    {
        double EE = NAN, MM = NAN;
        caps_t *z = caps_init(1.0, 0.001);
        caps_set_ldim(z, 12000);
        caps_logdetD0(z, 0, INFINITY, &EE, &MM, NULL);
        printf("xi0_EE %.17g\n", EE);
        printf("xi0_MM %.17g\n", MM);
        caps_free(z);
    }
    return 0;
}
