/*
 * Per-(element, mass) constants of the four muon DCS processes.
 *
 * The reference recomputes these inside every scalar call (three pow() per
 * bremsstrahlung evaluation, physics.hh:126-128; pow(Z, 1/3) per pair
 * production evaluation, dcs.hh:154; log(A) per DRSS call, dcs.hh:313-315).
 * Here the host computes them once per launch with the same libm calls and the
 * same operation order, so the values are bit-identical to the ones the
 * reference's CPU path uses, and the kernels read them from the launch
 * parameters (constant bank, warp-uniform).
 *
 * Host code that fills this struct must be compiled with -ffp-contract=off so
 * that no product is fused into an addition the reference rounds separately.
 */
#pragma once

#include <math.h>
#include <stdint.h>
#include <string.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Physical constants, physics.hh:54-58, 76. */
#define NOA_AVOGADRO_NUMBER 6.02214076E+23
#define NOA_ELECTRON_MASS 0.510998910E-03
#define NOA_MUON_MASS 0.10565839
#define NOA_X_FRACTION 5E-02

typedef struct noa_dcs_consts {
    /* element and particle */
    double A;
    double I;
    double mass;
    double Zd;      /* (double) Z */
    int32_t Z;
    int32_t pad_;
    double inv_mass;        /* 1 / mass */
    double inv_m2;          /* 1 / (mass mass) */
    double scale_A;         /* 1e3 N_A / A: the macroscopic factor of every process */

    /* bremsstrahlung, physics.hh:119-133 */
    double br_phie_factor;  /* mass / (me me sqrte) */
    double br_BZ_n;         /* Z==1 ? 202.4 : 182.7 Z^-1/3 */
    double br_BZ_e;         /* Z==1 ? 446   : 1429 Z^-2/3 */
    double br_D_n;          /* 1.54 A^0.27 */
    double br_dcs_factor;   /* 7.297182e-7 rem rem Z */
    double br_scale;        /* br_dcs_factor scale_A (FP32C final scaling) */
    double br_half_m2;      /* 0.5 mass mass */
    double br_Dn_sqrte_m2;  /* D_n sqrte - 2 */
    double br_BZe_mass;     /* BZ_e mass */

    /* pair production, dcs.hh:148-170 */
    double pp_Z13;          /* Z^(1/3) */
    double pp_kmax_shift;   /* mass (1 - 0.75 sqrte Z13) */
    double pp_r;            /* mass / me */
    double pp_AZ13;         /* A_ / Z13 */
    double pp_cL;           /* 2 sqrte me AZ13 */
    double pp_cLe;          /* 2.25 Z13 Z13 / (r r) */
    double pp_half_r2;      /* 0.5 r r */
    double pp_r2;           /* r r */
    double pp_inv_r2;       /* 1 / (r r) */
    double pp_r_AZ13;       /* r AZ13 */
    double pp_15_Z13;       /* 1.5 Z13 */
    double pp_cZ;           /* 1.794664e-34 Z */
    double pp_gamma1;       /* form-factor constants, dcs.hh:235-241 */
    double pp_gamma2;

    /* photonuclear, dcs.hh:310-319, 370-375 */
    double ph_logA;         /* log(A) */
    double ph_a_low;        /* exp(-0.1 log A), x < 0.0014 branch */
    double ph_q_min;        /* mpi (1 + 0.5 mpi / M) */
    double ph_log_q02;      /* log(Q02 / Lambda2), ALLM */
    double ph_inv_log_q02;  /* 1 / log(Q02 / Lambda2) */
    double ph_scale;        /* 0.5 cf 1e3 N_A / A, cf = 2.603096e-35 (FP32C final scaling) */

    /* ionisation, dcs.hh:408-443 */
    double io_Wmin;         /* 0.62 I */
    double io_k_rad;        /* 0.5 m1 m1 / me, radiative-correction threshold */
    double io_cZA;          /* 1.535336e-5 Z / A */

    /* float pairs (hi + lo to ~2^-48) for float-float arithmetic */
    float inv_mass_h, inv_mass_l;  /* 1 / mass */
    float mass_h, mass_l;          /* mass */
    float io_cm_h, io_cm_l;        /* (mass + me)^2: W_max = 2 me K (K + 2 mass) / ((mass + me)^2 + 2 me K) */
    float mass2_f;                 /* mass^2 rounded to float */
    float pp_kmax_shift_f;         /* pp_kmax_shift rounded to float */
    float ph_q_min_f;              /* ph_q_min rounded to float */
} noa_dcs_consts;

/* Fills c from (A, I, Z, mass) with the reference's expressions (host code;
 * compile with -ffp-contract=off). */
static inline void noa_dcs_fill_consts(noa_dcs_consts *c, double A, double I, int32_t Z, double mass) {
    memset(c, 0, sizeof *c);
    const double me = NOA_ELECTRON_MASS;
    c->A = A;
    c->I = I;
    c->mass = mass;
    c->Z = Z;
    c->Zd = (double)Z;
    c->inv_mass = 1. / mass;
    c->inv_mass_h = (float)c->inv_mass;
    c->inv_mass_l = (float)(c->inv_mass - (double)c->inv_mass_h);
    c->mass_h = (float)mass;
    c->mass_l = (float)(mass - (double)c->mass_h);
    {
        const double cm = (mass + me) * (mass + me);
        c->io_cm_h = (float)cm;
        c->io_cm_l = (float)(cm - (double)c->io_cm_h);
    }
    c->mass2_f = (float)(mass * mass);
    c->inv_m2 = 1. / (mass * mass);
    c->scale_A = 1E+03 * NOA_AVOGADRO_NUMBER / A;
    { // physics.hh:121-133
        const double sqrte = 1.648721271;
        c->br_phie_factor = mass / (me * me * sqrte);
        const double rem = 5.63588E-13 * me / mass;
        c->br_BZ_n = (Z == 1) ? 202.4 : 182.7 * pow((double)Z, -1. / 3.);
        c->br_BZ_e = (Z == 1) ? 446. : 1429. * pow((double)Z, -2. / 3.);
        c->br_D_n = 1.54 * pow(A, 0.27);
        c->br_dcs_factor = 7.297182E-07 * rem * rem * (double)Z;
        c->br_scale = c->br_dcs_factor * c->scale_A;
        c->br_half_m2 = 0.5 * mass * mass;
        c->br_Dn_sqrte_m2 = c->br_D_n * sqrte - 2.;
        c->br_BZe_mass = c->br_BZ_e * mass;
    }
    { // dcs.hh:153-166, 235-241
        const double sqrte = 1.6487212707;
        const double Z13 = pow((double)Z, 1. / 3.);
        c->pp_Z13 = Z13;
        c->pp_kmax_shift = mass * (1. - 0.75 * sqrte * Z13);
        c->pp_kmax_shift_f = (float)c->pp_kmax_shift;
        const double r = mass / me;
        c->pp_r = r;
        const double A_ = (Z == 1) ? 202.4 : 183.;
        c->pp_AZ13 = A_ / Z13;
        c->pp_cL = 2. * sqrte * me * c->pp_AZ13;
        c->pp_cLe = 2.25 * Z13 * Z13 / (r * r);
        c->pp_half_r2 = 0.5 * r * r;
        c->pp_r2 = r * r;
        c->pp_inv_r2 = 1. / (r * r);
        c->pp_r_AZ13 = r * c->pp_AZ13;
        c->pp_15_Z13 = 1.5 * Z13;
        c->pp_cZ = 1.794664E-34 * (double)Z;
        c->pp_gamma1 = (Z == 1) ? 4.4E-05 : 1.95E-05;
        c->pp_gamma2 = (Z == 1) ? 4.8E-05 : 5.30E-05;
    }
    { // dcs.hh:290, 313-315, 370-374
        const double M = 0.931494, mpi = 0.134977;
        c->ph_logA = log(A);
        c->ph_a_low = exp(-0.1 * log(A));
        c->ph_q_min = mpi * (1.0 + 0.5 * mpi / M);
        c->ph_q_min_f = (float)c->ph_q_min;
        c->ph_log_q02 = log(0.52544 / 0.06527);
        c->ph_inv_log_q02 = 1. / c->ph_log_q02;
        c->ph_scale = 0.5 * 2.603096E-35 * c->scale_A;
    }
    { // dcs.hh:422, 435-436
        c->io_Wmin = 0.62 * I;
        const double m1 = mass - me;
        c->io_k_rad = 0.5 * m1 * m1 / me;
        c->io_cZA = 1.535336E-05 * (double)Z / A;
    }
}

#ifdef __cplusplus
}
#endif
