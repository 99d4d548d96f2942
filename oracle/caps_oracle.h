/*
 * caps_oracle.h -- CPU restatement of the CaPS v0.5 logdetD path.
 * TEST INFRASTRUCTURE ONLY: the parity reference and the CPU baseline.
 */
#ifndef CAPS_ORACLE_H
#define CAPS_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

enum { ORACLE_PERFECT = 0, ORACLE_DRUDE = 1 };

/* dielectric model: perfect reflector, or Drude eps-1 = wp^2/(xi(xi+gamma)) (rad/s);
 * gamma = 0 gives the plasma model */
typedef struct { int kind; double omegap, gamma; } oracle_material_t;

typedef struct {
    double R, L;   /* sphere radius, separation (m) */
    int ldim;
    oracle_material_t plate, sphere;
} oracle_geom_t;

double oracle_logi(unsigned n);
double oracle_lfac(unsigned n);
double oracle_ratioI(double nu, double x);
double oracle_logI_asymp(double nu, double x);
double oracle_logK_asymp(double nu, double x);
void   oracle_logIK_half(int n, double x, double *logI, double *logK);
void   oracle_mie(double LbyR, double xi_, int l, double epsm1, double *lna, double *lnb);
double oracle_lnLambda(int l1, int l2, int m);
int    oracle_lmin(double LbyR, int ldim, int m);
double oracle_lnPl(int l, double x);
double oracle_lnPlm(int l, int m, double x);
double oracle_Plm_cf(long l, long m, double x);
double oracle_epsm1(const oracle_material_t *mat, double xi);

double oracle_logdet_lu(double *A, int n);
double oracle_logdet_1mM(double *M, int n, int *path);
void   oracle_M_dense(const oracle_geom_t *g, double xi_, int m, double *M);
double oracle_logdetD(const oracle_geom_t *g, double xi_, int m);
void   oracle_K_table(const oracle_geom_t *g, double xi_, int m, int nu_lo, int nu_hi, double *logK_TE, double *logK_TM);
double oracle_I(const oracle_geom_t *g, double xi_, int m, int l1, int l2, int p, int *sign);

double oracle_ht_drude(double LbyR);
double oracle_logdetD0_MM(const oracle_geom_t *g, int m);
double oracle_ht_perf(const oracle_geom_t *g, double eps);
double oracle_plasma_I(int nu, double omegap_);
double oracle_logdetD0_MM_plasma(const oracle_geom_t *g, int m, double omegap);
double oracle_ht_plasma(const oracle_geom_t *g, double omegap, double eps);

double oracle_bessel_logI0(double x);
double oracle_bessel_logI1(double x);
double oracle_bessel_logK0(double x);
double oracle_bessel_logK1(double x);
double oracle_bessel_logIn(int n, double x);
double oracle_bessel_logKn(int n, double x);
double oracle_capc_logdet(double R, double d, int lmax, double q, char DN, int hodlr);

void   oracle_logdetD_batch(const oracle_geom_t *g, int n, const double *xi, const int *m, double *out, int nthreads);
double oracle_free_energy(const oracle_geom_t *g, double T, double cutoff, double epsrel, int nthreads,
                          double *xi_out, double *v_out, int *nxi, int *ndet);

#ifdef __cplusplus
}
#endif
#endif
