/*
 * gp_internal.h -- device image of the physics tables and engine internals.
 *
 * The tables of `struct pumas_physics` (pumas.c:660-806) are copied to one
 * device allocation with the reference's row layouts: FP64 rows of
 * n_energies values indexed as [scheme][material][row] or [material][row],
 * and the FP32 DCS tables as [process][element][row][n_table_dcs][2]. At
 * 1.8 MB for four materials the whole image stays resident in the 129 MB L2
 * and its hot rows in L1.
 *
 * Per element constants that the reference recomputes inside the stepping
 * (screening exponents of Salvat et al., nuclear radii, Z^1/3, radiation
 * logarithms, pow(A, 0.27), ...) are evaluated once on the host at upload
 * time with the same expressions, which removes FP64 work from the device
 * and keeps the host libm values of the reference.
 */
#ifndef GP_INTERNAL_H
#define GP_INTERNAL_H

#include <stdint.h>

#define GP_N_DEL 4
#define GP_MAX_COMPONENTS 8

/* Per element constants. */
struct gp_element {
        double Z, A, I;
        int index;          /* element index in the DCS tables */
        int n_screen;       /* number of atomic screening terms, 1 to 3 */
        double amplitude[3];/* Salvat amplitudes (pumas.c:7348-7365) */
        double a_screen[3]; /* exponent / BOHR_RADIUS (pumas.c:7369) */
        double RN;          /* data_nuclear_radius (pumas.c:7143-7175) */
        double Ma;          /* Z M_p + (A - Z) M_n (pumas.c:7495) */
        double z13;         /* pow(Z, 1/3) */
        double z13_inv;     /* 1 / pow(Z, 1/3) (SSR bremsstrahlung) */
        double zm13;        /* pow(Z, -1/3) (SSR pair production) */
        double z23;         /* pow(Z, 2/3) */
        double dn;          /* 1.54 pow(A, 0.27) */
        double rad_log;     /* radiation_logarithm(Z) */
        double qmax_m_pair; /* 1 - 0.75 sqrt(e) Z^1/3, pair range */
        double qmax_m_brems;/* 1 - 0.75 SQRTE Z^1/3, SSR brems bound */
        double muni;        /* (m RN / hbar c)^2 / 6, polar brems */
        double mu_qc;       /* SSR bremsstrahlung nuclear factor */
        double ssr_delta1;  /* SSR bremsstrahlung delta1(mu_qc) */
        double ssr_delta2;  /* SSR bremsstrahlung delta2(mu_qc) */
        double pair_pref;   /* 4 / (3 pi) Z (alpha_em r_e)^2, SSR pairs */
        double pair_medn2;  /* (m_e / m d_n)^2, SSR pairs (MeV units) */
        double log_A;       /* log(A), DRSS shadowing */
        double shadow_low;  /* exp(-0.1 log(A)), DRSS shadowing */
};

/* Numerical constants evaluated on the host with the reference's
 * expressions (constant folded or libm). */
struct gp_constants {
        double exp1;        /* exp(1.) */
        double exp_half;    /* exp(0.5) */
        double exp_m16;     /* exp(-1. / 6.) */
        double exp_13;      /* exp(1. / 3.) */
        double exp_m13;     /* exp(-1. / 3.) */
        double allm_lq0;    /* log(Q02 / Lambda2) in ALLM97 */
        double pair_me_m2;  /* pow(ME / m, 2.) with m in MeV, SSR pairs */
};

/* Bucket index of a monotone table: for a non-negative double v with raw
 * bits b, bucket (b >> GP_LUT_SHIFT) - key0 (an 8 bit mantissa slice of a
 * binade) holds the largest row i with table[i] below the bucket's lower
 * edge. A lookup then needs one load and at most a few integer compares
 * instead of a bisection (table_index, pumas.c:4174-4233); the row found
 * is the same. */
#define GP_LUT_SHIFT 44
struct gp_lut {
        int key0;
        int n;
        const unsigned short * idx;
};

/* Identifiers of the searched tables: the energy grid K, then per scheme
 * and material the grammage X and proper time T, per material the DEL
 * interaction lengths NI_in and per scheme and material the EHS ones. */
#define GP_LUT_K 0
#define GP_LUT_X(T_, s, m) (1 + (s) * (T_).n_materials + (m))
#define GP_LUT_T(T_, s, m) (1 + (2 + (s)) * (T_).n_materials + (m))
#define GP_LUT_NI_IN(T_, m) (1 + 4 * (T_).n_materials + (m))
#define GP_LUT_NI_EL(T_, s, m) (1 + (5 + (s)) * (T_).n_materials + (m))
#define GP_N_LUT(n_materials) (1 + 7 * (n_materials))

/* Baked cubic Hermite interpolants. For a table (grid x, values y,
 * derivatives m) the reference computes, at each lookup in row i
 * (table_interpolate_pchip and math_pchip_interpolate, pumas.c:4118-4157),
 * dx = x[i+1] - x[i], m0 = m[i] dx, m1 = m[i+1] dx (m0 in row 0), then
 * c2 = -3 (y[i] - y[i+1]) - 2 m0 - m1 and c3 = 2 (y[i] - y[i+1]) + m0 + m1.
 * These are evaluated once on the host with the same expressions and
 * stored per row; a lookup is then p0 + t (m0 + t (c2 + t c3)), each
 * product and sum rounded on its own as in the reference, with
 * t = (v - x[i]) / dx. The quotient is the correctly rounded one, obtained
 * from the stored 1 / dx with one residual correction (Markstein): q0 =
 * (v - x[i]) (1 / dx), r = (v - x[i]) - q0 dx exactly by a fused
 * multiply-add, t = q0 + r (1 / dx) rounded once. */
struct __align__(32) gp_coef {
        double p0, m0, c2, c3;
};
struct __align__(32) gp_node {
        double x, inv_dx, dx, pad;
};

/* Identifiers of the baked interpolants, M materials, s a scheme in {0, 1}
 * (CSDA, MIXED) and s3 the Ms1 scheme row in {0, 1, 2}. Node grids use the
 * GP_LUT_* identifiers. */
#define GP_C_X(M, s, m) ((s) * (M) + (m))
#define GP_C_T(M, s, m) ((2 + (s)) * (M) + (m))
#define GP_C_DE(M, s, m) ((4 + (s)) * (M) + (m))
#define GP_C_OMEGA(M, m) (6 * (M) + (m))
#define GP_C_CS(M, m) (7 * (M) + (m))
#define GP_C_NI_IN(M, m) (8 * (M) + (m))
#define GP_C_NI_EL(M, s, m) ((9 + (s)) * (M) + (m))
#define GP_C_MU0(M, m) (11 * (M) + (m))
#define GP_C_MS1(M, s3, m) ((12 + (s3)) * (M) + (m))
#define GP_C_K_OF_X(M, s, m) ((15 + (s)) * (M) + (m))
#define GP_C_X_OF_T(M, s, m) ((17 + (s)) * (M) + (m))
#define GP_C_K_OF_NI_IN(M, m) (19 * (M) + (m))
#define GP_C_K_OF_NI_EL(M, s, m) ((20 + (s)) * (M) + (m))
#define GP_N_COEF(M) (22 * (M))

struct gp_tables {
        int n_energies, n_materials, n_elements, n_components, n_table_dcs;
        /* DCS models (struct pumas_physics_settings, pumas.h:742-771):
         * bremsstrahlung 0 SSR, 1 KKP, 2 ABB; pair production 0 SSR,
         * 1 KKP; photonuclear 0 DRSS, 1 BBKS, 2 BM. */
        int model_brems, model_pair, model_photo;
        double ctau, mass, cutoff, elastic_ratio;
        const double *K, *K_dX, *K_dNI_in, *K_dNI_el;
        const double *X, *X_dK, *X_dT, *T, *T_dK, *dE, *dE_dK;
        const double *Omega, *Omega_dK, *NI_el, *NI_el_dK, *NI_in, *NI_in_dK;
        const double *CS, *CS_dK, *CSf, *CSf_dK, *CSn, *CSn_dK;
        const float *DCS, *DCS_x, *DCS_env;
        const double *Kt, *a_max, *b_max, *Mu0, *Mu0_dK, *Lb, *Lb_dK;
        const double *Ms1, *Ms1_dK;
        const double * Li; /* CSDA magnetic moments, 8 orders per material */
        const int * elements_in;
        const int * comp_start;
        const int * comp_element;
        const double * comp_fraction;
        const double * material_density;
        const struct gp_element * element;
        const struct gp_lut * lut;
        const struct gp_coef * coef; /* GP_N_COEF tables of n_energies rows */
        const struct gp_node * node; /* GP_N_LUT grids of n_energies rows */
        struct gp_constants k;
};

/* Host side handle. */
struct gpumas_physics {
        struct gp_tables tables; /* device pointers */
        void * device_blob;
        size_t device_size;
        int n_materials;
        int n_elements;
        int particle; /* enum pumas_particle: 0 muon, 1 tau */
        char ** material_name;
        int device;
};

#ifdef __cplusplus
extern "C" {
#endif
int gp_physics_tables(const struct gpumas_physics * physics,
    struct gp_tables * tables);
/* Reserve the static slot pool of the allocation free entry point on the
 * current device (gp_batch.cu). */
int gp_static_reserve(void);
#ifdef __cplusplus
}
#endif

#endif
