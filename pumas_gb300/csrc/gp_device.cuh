/*
 * gp_device.cuh -- device side muon transport physics for sm_103a.
 *
 * A GPU restatement of the reference transport (PUMAS 1.2.3, src/pumas.c):
 * table interpolants, CEL / DEL / EHS samplers, Coulomb scattering, the
 * default DCS models and the polar angle samplers. Floating point
 * expressions keep the reference's evaluation order. Logarithms and
 * exponentials are the engine's table-driven ones (gp_math.cuh, below one
 * ulp, equal to glibc's in about 98 % of arguments); the other CUDA double
 * precision functions differ from glibc by at most an ulp or two. The
 * parity tests bound the effect. Differences in structure, all result
 * preserving:
 *
 *   - no per context index cache in table lookups (pumas.c:4174-4210): the
 *     cache never changes the bracketing index;
 *   - per element constants come precomputed from the host (gp_internal.h);
 *   - the FP32 DCS interpolation (pumas.c:11276-11346) uses
 *     (float)log((double)x) and (float)exp((double)x), which agree with
 *     glibc's logf / expf far more often than CUDA's single precision ones;
 *   - the x87 extended precision of the Coulomb pole reduction
 *     (pumas.c:7524-7683) is replaced by double precision. It only enters
 *     the choice of the hard scatterer in compound materials and is skipped
 *     altogether for single element ones, where the choice is forced;
 *   - every rejection loop, unbounded in the reference (pumas.c:5839, 6115,
 *     6241, 6918, 6973, 11208), has an iteration cap after which the event
 *     stops with PUMAS_RETURN_INTERNAL_ERROR, so that no GPU thread can
 *     spin forever.
 */
#ifndef GP_DEVICE_CUH
#define GP_DEVICE_CUH

#include <stdint.h>

#include "gp_math.cuh"
#include "gp_libmf.cuh"
#include "gp_models.cuh"

#include "gpumas.h"
#include "gp_internal.h"

#define GP_EPSILON_X 3E-03
#define GP_STEP_MIN 1E-07
#define GP_ALPHA_EM 7.2973525693E-03
#define GP_HBAR_C 1.973269804E-16
#define GP_ELECTRON_MASS 0.510998910E-03
#define GP_ELECTRON_RADIUS 2.817940285E-15
#define GP_PROTON_MASS 0.938272
#define GP_NEUTRON_MASS 0.939565
#define GP_PION_MASS 0.13957018
#define GP_AVOGADRO 6.02214076E+23
#define GP_PI 3.14159265358979323846
/* FLT_EPSILON of the reference, a float literal: exactly 2^-23. */
#define GP_FLT_EPSILON 0x1p-23
/* Larmor factor in m^-1 GeV/c T^-1 (pumas.c:145-150). */
#define GP_LARMOR_FACTOR 0.299792458
#define GP_DBL_EPSILON 2.2204460492503131E-16
#define GP_DBL_MAX 1.7976931348623157E+308

/* Default iteration cap of the reference's unbounded rejection loops
 * (gp_config.max_trials, gpumas_context_trials_set). */
#define GP_MAX_REJECTIONS_DEFAULT 100000

#define GPD static __device__ __forceinline__

/* Products and sums rounded separately, as on the host. The library is
 * built without contraction (--fmad=false) anyway; these mark the places
 * where the reference's expression cancels and a fused multiply-add would
 * change the result beyond the parity tolerance. */
#define GP_MUL(a, b) __dmul_rn((a), (b))
#define GP_ADD(a, b) __dadd_rn((a), (b))
#define GP_SUB(a, b) __dsub_rn((a), (b))

/* Transport settings of a launch (the public fields of pumas_context). */
struct gp_config {
        int energy_loss, decay, direction, scattering;
        int event;
        double limit_energy, limit_distance, limit_grammage, limit_time;
        double accuracy;
        uint64_t seed;
        /* Trials of a rejection sampling before the event fails with
         * GPUMAS_RETURN_INTERNAL_ERROR (GP_MAX_REJECTIONS_DEFAULT by
         * default). */
        int max_trials;
        /* Events continue the random stream and Box-Muller cache of their
         * previous call, read from their result entry (gpumas_result). */
        int carry;
};

/* ------------------------------------------------------------------------ */
/* Philox-4x32-10 stream, keyed by (seed, event id): draw n of an event     */
/* uses block n / 2 of counter (block, 0, event), 64 bits per draw mapped   */
/* to ((w >> 12) + 0.5) 2^-52.                                              */
/* ------------------------------------------------------------------------ */
GPD void gp_philox(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3,
    uint32_t k0, uint32_t k1, uint32_t * out)
{
#pragma unroll
        for (int round = 0; round < 10; round++) {
                const uint32_t hi0 = __umulhi(0xD2511F53u, c0);
                const uint32_t lo0 = 0xD2511F53u * c0;
                const uint32_t hi1 = __umulhi(0xCD9E8D57u, c2);
                const uint32_t lo1 = 0xCD9E8D57u * c2;
                c0 = hi1 ^ c1 ^ k0;
                c1 = lo1;
                c2 = hi0 ^ c3 ^ k1;
                c3 = lo0;
                k0 += 0x9E3779B9u;
                k1 += 0xBB67AE85u;
        }
        out[0] = c0;
        out[1] = c1;
        out[2] = c2;
        out[3] = c3;
}

/* Exact map of a 64 bit word to ]0, 1[: 1.m - (1 - 2^-53). */
GPD double gp_word_to_uniform(uint32_t lo, uint32_t hi)
{
        const uint64_t w = ((uint64_t)hi << 32) | lo;
        const double one_m = __longlong_as_double(
            (long long)(0x3FF0000000000000ull | (w >> 12)));
        return __dsub_rn(one_m, 0x1.fffffffffffffp-1);
}

/* Per event state: the pumas_state, the per event part of the reference's
 * simulation_context (pumas.c:426-477) and the random stream. */
struct gp_event {
        double charge, energy, distance, grammage, time, weight;
        double pos[3], dir[3];
        int decayed;
        int step_first, step_event, step_foreseen;
        double step_X_limit, step_invlb1;
        int randn_done;
        double randn_next;
        double lifetime;
        uint64_t id;
        uint32_t n;
        double rnext;
        uint32_t k0, k1;
        int steps;
        int status;
};

/* Recorder of one event (struct pumas_recorder, pumas.h:432-458): the
 * event's frame array of a gpumas_recorder and the count of frames the
 * reference would have recorded so far. Transport functions take a
 * pointer to it that is NULL when not recording; they are inlined, so the
 * recording code vanishes from kernels that never record. */
struct gp_rec {
        gpumas_frame * frames;
        int max_frames;
        int period;
        int count;
};

/* record_state (pumas.c:7738-7780) into the event's frame array. */
GPD void gp_rec_frame(gp_rec * r, const gp_event & e, int medium, int event)
{
        if (r->count < r->max_frames) {
                gpumas_frame & f = r->frames[r->count];
                f.state.charge = e.charge;
                f.state.energy = e.energy;
                f.state.distance = e.distance;
                f.state.grammage = e.grammage;
                f.state.time = e.time;
                f.state.weight = e.weight;
                for (int k = 0; k < 3; k++) {
                        f.state.position[k] = e.pos[k];
                        f.state.direction[k] = e.dir[k];
                }
                f.state.decayed = e.decayed;
                f.medium = medium;
                f.event = event;
        }
        r->count++;
}

GPD double gp_random(gp_event & e)
{
        double u;
        if (e.n & 1u) {
                u = e.rnext;
        } else {
                uint32_t x[4];
                gp_philox(e.n >> 1, 0u, (uint32_t)e.id,
                    (uint32_t)(e.id >> 32), e.k0, e.k1, x);
                u = gp_word_to_uniform(x[0], x[1]);
                e.rnext = gp_word_to_uniform(x[2], x[3]);
        }
        e.n++;
        return u;
}

/* ------------------------------------------------------------------------ */
/* Tables (pumas.c:3644-4752).                                              */
/* ------------------------------------------------------------------------ */
GPD int gp_sch(int scheme) { return (scheme > 1) ? 1 : scheme; }
GPD int gp_sch_el(int scheme) { return (scheme >= 1) ? 1 : 0; }

/* table_index (pumas.c:4174-4233): the row i with table[i] <= value <
 * table[i + 1], through the table's bucket index (gp_lut). Rows are
 * non-negative, so values are compared through their raw bits on the
 * integer pipes. */
GPD int gp_index(const gp_tables & T, int lut_id,
    const double * __restrict__ table, double value)
{
        const int imax = T.n_energies - 1;
        if (value < __ldg(table)) return -1;
        if (value >= __ldg(table + imax)) return imax;
        const gp_lut & L = T.lut[lut_id];
        const int n = L.n;
        if (n > 0) {
                const long long vb = __double_as_longlong(value);
                const int k = (int)(vb >> GP_LUT_SHIFT) - L.key0;
                int i = (k < 0) ? 0 : (k >= n) ? imax - 1 : (int)__ldg(L.idx + k);
                while ((i + 1 < imax) &&
                    (vb >= __double_as_longlong(__ldg(table + i + 1))))
                        i++;
                return i;
        }
        int i1 = 0, i2 = imax;
        do {
                const int i3 = (i1 + i2) >> 1;
                if (value >= __ldg(table + i3))
                        i1 = i3;
                else
                        i2 = i3;
        } while (i2 - i1 >= 2);
        return i1;
}

/* The correctly rounded quotient a / b from rb = 1 / b (correctly rounded):
 * one residual correction of q0 = a rb, with the residual a - q0 b exact
 * by a fused multiply-add (Markstein, IBM J. Res. Dev. 34 (1990) 111). */
GPD double gp_quotient(double a, double b, double rb)
{
        const double q0 = GP_MUL(a, rb);
        return fma(fma(-q0, b, a), rb, q0);
}

/* The cubic p0 + t (m0 + t (c2 + t c3)), every product and sum rounded on
 * its own as in the reference's C code. */
GPD double gp_horner3(double t, double p0, double m0, double c2, double c3)
{
        return GP_ADD(p0, GP_MUL(t, GP_ADD(m0, GP_MUL(t, GP_ADD(c2,
            GP_MUL(t, c3))))));
}

/* math_pchip_interpolate (pumas.c:4118-4125). */
GPD double gp_pchip(double t, double p0, double p1, double m0, double m1)
{
        const double d = GP_SUB(p0, p1);
        const double c2 =
            GP_SUB(GP_SUB(GP_MUL(-3., d), GP_MUL(2., m0)), m1);
        const double c3 = GP_ADD(GP_ADD(GP_MUL(2., d), m0), m1);
        return gp_horner3(t, p0, m0, c2, c3);
}

/* table_interpolate_pchip (pumas.c:4146-4157). */
GPD double gp_interpolate(const gp_tables & T, int lut_id,
    const double * __restrict__ X, const double * __restrict__ Y,
    const double * __restrict__ M, double x)
{
        const int i1 = gp_index(T, lut_id, X, x);
        const int i2 = i1 + 1;
        const double x1 = __ldg(X + i1);
        const double dX = GP_SUB(__ldg(X + i2), x1);
        const double t = __ddiv_rn(GP_SUB(x, x1), dX);
        const double m1 = GP_MUL(__ldg(M + i1), dX);
        const double m2 = (i2 > 1) ? GP_MUL(__ldg(M + i2), dX) : m1;
        return gp_pchip(t, __ldg(Y + i1), __ldg(Y + i2), m1, m2);
}

/* Baked cubic Hermite interpolant (gp_coef, gp_node): the same rows and
 * coefficients as table_interpolate_pchip (pumas.c:4146-4157). */
GPD double gp_baked_row(const gp_tables & T, int grid, int cid, int i,
    double x)
{
        const size_t ne = (size_t)T.n_energies;
        const double2 * n = (const double2 *)(T.node + grid * ne + i);
        const double2 nd = __ldg(n);
        const double t = gp_quotient(GP_SUB(x, nd.x), __ldg(&n[1].x), nd.y);
        const double2 * c = (const double2 *)(T.coef + cid * ne + i);
        const double2 c01 = __ldg(c);
        const double2 c23 = __ldg(c + 1);
        return gp_horner3(t, c01.x, c01.y, c23.x, c23.y);
}

GPD double gp_baked(const gp_tables & T, int grid,
    const double * __restrict__ gx, int cid, double x)
{
        return gp_baked_row(T, grid, cid, gp_index(T, grid, gx, x), x);
}

#define GP_ROW(s, m) ((long)((s) * T.n_materials + (m)) * T.n_energies)
#define GP_MROW(m) ((long)(m) * T.n_energies)

GPD double gp_cel_grammage(
    const gp_tables & T, int scheme, int material, double kinetic)
{
        const int imax = T.n_energies - 1;
        if (kinetic < __ldg(T.K)) return 0.;
        const int s = gp_sch(scheme);
        if (kinetic >= __ldg(T.K + imax)) {
                const double a = __ldg(T.a_max + material);
                const double b = __ldg(T.b_max + s * T.n_materials + material);
                const double K0 = __ldg(T.K + imax);
                const double K1 = a / b + T.mass;
                return __ldg(T.X + GP_ROW(s, material) + imax) +
                    1. / b * gp_log((kinetic + K1) / (K0 + K1));
        }
        return gp_baked(T, GP_LUT_K, T.K, GP_C_X(T.n_materials, s, material),
            kinetic);
}

GPD double gp_cel_grammage_as_time(
    const gp_tables & T, int scheme, int material, double time)
{
        const int imax = T.n_energies - 1;
        const int s = gp_sch(scheme);
        const double * Tt = T.T + GP_ROW(s, material);
        if (time < __ldg(Tt)) return 0.;
        if (time >= __ldg(Tt + imax)) {
                const double a = __ldg(T.a_max + material);
                const double b = __ldg(T.b_max + s * T.n_materials + material);
                const double E0 = __ldg(T.K + imax) + T.mass;
                const double tmax = __ldg(Tt + imax);
                const double r =
                    E0 / (a + b * E0) * gp_exp(a * (time - tmax) / T.mass);
                const double kinetic = a * r / (1. - b * r) - T.mass;
                const double K1 = a / b + T.mass;
                return __ldg(T.X + GP_ROW(s, material) + imax) +
                    1. / b * gp_log((kinetic + K1) / (E0 - T.mass + K1));
        }
        return gp_baked(T, GP_LUT_T(T, s, material), Tt,
            GP_C_X_OF_T(T.n_materials, s, material), time);
}

GPD double gp_cel_proper_time(
    const gp_tables & T, int scheme, int material, double kinetic)
{
        const int imax = T.n_energies - 1;
        if (kinetic < __ldg(T.K)) return 0.;
        const int s = gp_sch(scheme);
        if (kinetic >= __ldg(T.K + imax)) {
                const double a = __ldg(T.a_max + material);
                const double b = __ldg(T.b_max + s * T.n_materials + material);
                const double E0 = __ldg(T.K + imax) + T.mass;
                const double E1 = kinetic + T.mass;
                return __ldg(T.T + GP_ROW(s, material) + imax) +
                    T.mass / a * gp_log((E1 / E0) * (a + b * E0) / (a + b * E1));
        }
        return gp_baked(T, GP_LUT_K, T.K, GP_C_T(T.n_materials, s, material),
            kinetic);
}

GPD double gp_cel_kinetic_energy(
    const gp_tables & T, int scheme, int material, double grammage)
{
        const int imax = T.n_energies - 1;
        const int s = gp_sch(scheme);
        const double * X = T.X + GP_ROW(s, material);
        if (grammage < __ldg(X)) return 0.;
        if (grammage >= __ldg(X + imax)) {
                const double a = __ldg(T.a_max + material);
                const double b = __ldg(T.b_max + s * T.n_materials + material);
                const double K0 = __ldg(T.K + imax);
                const double K1 = a / b + T.mass;
                return (K0 + K1) * gp_exp(b * (grammage - __ldg(X + imax))) - K1;
        }
        return gp_baked(T, GP_LUT_X(T, s, material), X,
            GP_C_K_OF_X(T.n_materials, s, material), grammage);
}

GPD double gp_cel_energy_loss(
    const gp_tables & T, int scheme, int material, double kinetic)
{
        const int imax = T.n_energies - 1;
        if (kinetic < __ldg(T.K)) return 0.;
        const int s = gp_sch(scheme);
        if (kinetic >= __ldg(T.K + imax)) {
                return __ldg(T.a_max + material) +
                    __ldg(T.b_max + s * T.n_materials + material) *
                    (kinetic + T.mass);
        }
        return gp_baked(T, GP_LUT_K, T.K,
            GP_C_DE(T.n_materials, s, material), kinetic);
}

GPD double gp_cel_straggling(const gp_tables & T, int material, double kinetic)
{
        const int imax = T.n_energies - 1;
        if (kinetic < __ldg(T.K)) return 0.;
        const double Kmax = __ldg(T.K + imax);
        if (kinetic >= Kmax) {
                const double r = (kinetic + T.mass) / (Kmax + T.mass);
                return __ldg(T.Omega + GP_MROW(material) + imax) * r * r;
        }
        return gp_baked(T, GP_LUT_K, T.K, GP_C_OMEGA(T.n_materials, material),
            kinetic);
}

GPD double gp_del_cross_section(
    const gp_tables & T, int material, double kinetic)
{
        const int imax = T.n_energies - 1;
        if (kinetic < __ldg(T.K)) return 0.;
        if (kinetic >= __ldg(T.K + imax))
                return __ldg(T.CS + GP_MROW(material) + imax);
        return gp_baked(T, GP_LUT_K, T.K, GP_C_CS(T.n_materials, material),
            kinetic);
}

GPD double gp_del_interaction_length(
    const gp_tables & T, int material, double kinetic)
{
        const int imax = T.n_energies - 1;
        if (kinetic < __ldg(T.K)) return 0.;
        if (kinetic >= __ldg(T.K + imax)) {
                const double k0 = __ldg(T.K + imax);
                const double a0 = __ldg(T.a_max + material);
                const double b0 = __ldg(T.b_max + T.n_materials + material);
                const double cs = __ldg(T.CS + GP_MROW(material) + imax);
                const double dZ =
                    cs / b0 * gp_log((a0 + b0 * (kinetic + T.mass)) /
                                  (a0 + b0 * (k0 + T.mass)));
                return __ldg(T.NI_in + GP_MROW(material) + imax) + dZ;
        }
        return gp_baked(T, GP_LUT_K, T.K, GP_C_NI_IN(T.n_materials, material),
            kinetic);
}

GPD double gp_del_kinetic_from_interaction_length(
    const gp_tables & T, int material, double nI)
{
        const int imax = T.n_energies - 1;
        const double * NI = T.NI_in + GP_MROW(material);
        if (nI < __ldg(NI)) return 0.;
        if (nI >= __ldg(NI + imax)) {
                const double k0 = __ldg(T.K + imax);
                const double a0 = __ldg(T.a_max + material);
                const double b0 = __ldg(T.b_max + T.n_materials + material);
                const double cs = __ldg(T.CS + GP_MROW(material) + imax);
                const double nI0 = __ldg(NI + imax);
                return ((a0 + b0 * (k0 + T.mass)) * gp_exp(b0 * (nI - nI0) / cs) -
                           a0) / b0 - T.mass;
        }
        return gp_baked(T, GP_LUT_NI_IN(T, material), NI,
            GP_C_K_OF_NI_IN(T.n_materials, material), nI);
}

GPD double gp_ehs_interaction_length(
    const gp_tables & T, int scheme, int material, double kinetic)
{
        const int imax = T.n_energies - 1;
        if (kinetic < __ldg(T.K)) return 0.;
        const double * NI = T.NI_el + GP_ROW(gp_sch_el(scheme), material);
        if (kinetic >= __ldg(T.K + imax)) {
                const double k0 = __ldg(T.K + imax - 1);
                const double k1 = __ldg(T.K + imax);
                const double nI0 = __ldg(NI + imax - 1);
                const double nI1 = __ldg(NI + imax);
                return nI1 + (kinetic - k1) * (nI1 - nI0) / (k1 - k0);
        }
        return gp_baked(T, GP_LUT_K, T.K,
            GP_C_NI_EL(T.n_materials, gp_sch_el(scheme), material), kinetic);
}

GPD double gp_ehs_kinetic_from_interaction_length(
    const gp_tables & T, int scheme, int material, double nI)
{
        const int imax = T.n_energies - 1;
        const double * NI = T.NI_el + GP_ROW(gp_sch_el(scheme), material);
        if (nI < __ldg(NI)) return 0.;
        if (nI >= __ldg(NI + imax)) {
                const double k0 = __ldg(T.K + imax - 1);
                const double k1 = __ldg(T.K + imax);
                const double nI0 = __ldg(NI + imax - 1);
                const double nI1 = __ldg(NI + imax);
                return k1 + (nI - nI1) * (k1 - k0) / (nI1 - nI0);
        }
        return gp_baked(T, GP_LUT_NI_EL(T, gp_sch_el(scheme), material), NI,
            GP_C_K_OF_NI_EL(T.n_materials, gp_sch_el(scheme), material), nI);
}

/* table_get_msc (pumas.c:4077-4111). */
GPD void gp_table_get_msc(const gp_tables & T, int energy_loss, int material,
    double kinetic, double & mu0, double & invlb1)
{
        const int imax = T.n_energies - 1;
        const int s = gp_sch(energy_loss);
        const double * Mu0 = T.Mu0 + GP_MROW(material);
        const double * Ms1 = T.Ms1 + GP_ROW(s + 1, material);
        const double K1 = __ldg(T.K + 1);
        if (kinetic < K1) {
                mu0 = __ldg(Mu0 + 1);
                invlb1 = __ldg(Ms1 + 1) * sqrt(K1 / kinetic);
        } else if (kinetic >= __ldg(T.K + imax)) {
                mu0 = __ldg(Mu0 + imax);
                invlb1 = __ldg(Ms1 + imax) * __ldg(T.K + imax) / kinetic;
        } else {
                const int i1 = gp_index(T, GP_LUT_K, T.K, kinetic);
                mu0 = gp_baked_row(T, GP_LUT_K, GP_C_MU0(T.n_materials,
                    material), i1, kinetic);
                invlb1 = gp_baked_row(T, GP_LUT_K, GP_C_MS1(T.n_materials,
                    s + 1, material), i1, kinetic);
        }
}

/* coulomb_ehs_length (pumas.c:7446-7466). */
GPD double gp_coulomb_ehs_length(
    const gp_tables & T, int material, double kinetic)
{
        const double p2 = kinetic * (kinetic + 2. * T.mass);
        const int imax = T.n_energies - 1;
        const double * Lb = T.Lb + GP_MROW(material);
        if (kinetic < __ldg(T.K + 1)) {
                return __ldg(Lb + 1) / p2;
        } else if (kinetic >= __ldg(T.K + imax)) {
                return __ldg(Lb + imax) / p2;
        } else {
                const int i1 = gp_index(T, GP_LUT_K, T.K, kinetic);
                const double2 * n = (const double2 *)(T.node + i1);
                const double2 nd = __ldg(n);
                const double h =
                    gp_quotient(GP_SUB(kinetic, nd.x), __ldg(&n[1].x), nd.y);
                const double l1 = __ldg(Lb + i1);
                return GP_ADD(l1, GP_MUL(h, GP_SUB(__ldg(Lb + i1 + 1), l1))) /
                    p2;
        }
}

/* ------------------------------------------------------------------------ */
/* Coulomb scattering (pumas.c:7203-7683).                                  */
/* ------------------------------------------------------------------------ */

/* coulomb_screening_parameters (pumas.c:7203-7387) with the element's
 * Salvat amplitudes and exponents from the host. The reference stores the
 * nuclear screening after the n atomic ones (screening[n]); here it is
 * returned in N, so that every array index is a constant once the loops
 * are unrolled and the arrays stay in registers. Returns n + 1. */
GPD int gp_coulomb_screening(const gp_element & el, double mass,
    double kinetic, double kinetic0, double * amplitude, double * screening,
    double & N)
{
        const double Z = el.Z;
        const double aZE = GP_ALPHA_EM * Z * (kinetic + mass);
        const double p2 = kinetic * (kinetic + 2. * mass);
        const double zeta2 = aZE * aZE / p2;
        double f;
        if (zeta2 < 1) {
                f = 1. / (1. + zeta2) + 0.20205690315959424 -
                    0.03692775514336999 * zeta2 +
                    0.008349277381922926 * zeta2 * zeta2;
                f *= zeta2;
        } else {
                const double r2i = 1. / (1. + zeta2);
                const double phi = -atan(sqrt(zeta2));
                f = -0.5 * gp_log(r2i) + 0.5 * (1. - r2i) +
                    1. / 12. * (1. - cos(2 * phi) * r2i) -
                    1. / 120. * (1. - cos(4 * phi) * r2i * r2i) +
                    1. / 252. * (1. - cos(6 * phi) * r2i * r2i * r2i);
        }
        const double ktv = gp_exp(2 * f);
        const double p02 = kinetic0 * (kinetic0 + 2. * mass);
        const double d = 0.25 * GP_HBAR_C * GP_HBAR_C / p02 * ktv;
        const int n = el.n_screen;
        for (int i = 0; i < 3; i++) {
                if (i < n) {
                        amplitude[i] = el.amplitude[i];
                        const double a = el.a_screen[i];
                        screening[i] = d * a * a;
                }
        }
        N = 12. * d / (el.RN * el.RN);
        return n + 1;
}

/* coulomb_nuclear_form_factor (pumas.c:7396-7416). */
GPD double gp_coulomb_nuclear_form_factor(double mu, double N)
{
        if (mu <= 0.)
                return 1.;
        else if (mu > 1.)
                return 0.;
        const double x2 = 10. * mu / N;
        double d;
        if (x2 <= 1E-04) {
                d = 1. / (1. + 0.1 * x2);
        } else {
                const double x = sqrt(x2);
                double sx, cx;
                sincos(x, &sx, &cx);
                d = 3 * (sx - x * cx) / (x2 * x);
        }
        return d * d;
}

/* coulomb_normalisation (pumas.c:7428-7435). */
GPD double gp_coulomb_normalisation(
    double Z, double A, double mass, double kinetic, double kinetic0)
{
        const double p2 = kinetic * (kinetic + 2. * mass);
        const double p02 = kinetic0 * (kinetic0 + 2. * mass);
        double d = GP_ALPHA_EM * Z * GP_HBAR_C * (kinetic + mass);
        return A * 1E-03 * p2 * p02 / (d * d * GP_PI * GP_AVOGADRO);
}

/* coulomb_spin_factor (pumas.c:7475-7479). */
GPD double gp_coulomb_spin_factor(double mass, double kinetic)
{
        const double e = kinetic + mass;
        return kinetic * (e + mass) / (e * e);
}

/* coulomb_frame_parameters (pumas.c:7492-7508). */
GPD void gp_coulomb_frame_parameters(double Ma, double mass, double kinetic,
    double & kinetic0, double * parameters)
{
        double M2 = mass + Ma;
        M2 *= M2;
        const double sCM12i = 1. / sqrt(M2 + 2. * Ma * kinetic);
        parameters[0] = (kinetic + mass + Ma) * sCM12i;
        kinetic0 = (kinetic * Ma + mass * (mass + Ma)) * sCM12i - mass;
        if (kinetic0 < 1E-09) kinetic0 = 1E-09;
        const double etot = kinetic + mass + Ma;
        const double betaCM2 = kinetic * (kinetic + 2. * mass) / (etot * etot);
        double rM2 = mass / Ma;
        rM2 *= rM2;
        parameters[1] = sqrt(rM2 * (1. - betaCM2) + betaCM2);
}

/* coulomb_pole_reduction (pumas.c:7524-7576), N = screening[n]. */
GPD void gp_coulomb_pole_reduction(int n_parameters, const double * amplitude,
    const double * screening, double N, double * a, double * b, double * c)
{
        const int n = n_parameters - 1;
        for (int i = 0; i < 3; i++) a[i] = b[i] = 0.;
        for (int i = 0; i < 4; i++) c[i] = 0.;
        for (int i = 0; i < 3; i++) {
                if (i >= n) break;
                const double Ai = amplitude[i];
                const double Bi = screening[i];
                b[i] = Ai * Ai;
                for (int j = i + 1; j < 3; j++) {
                        if (j >= n) break;
                        const double d =
                            2 * Ai * amplitude[j] / (screening[j] - Bi);
                        a[i] += d;
                        a[j] -= d;
                }
        }
        double Sa[4] = { 0, 0, 0, 0 }, Sb[4] = { 0, 0, 0, 0 };
        for (int i = 0; i < 3; i++) {
                if (i >= n) break;
                const double x = 1. - screening[i] / N;
                double r = x;
                for (int j = 0; j < 4; j++) {
                        Sa[j] += a[i] / r;
                        r *= x;
                        Sb[j] += b[i] / r;
                }
        }
        double tmp = 1;
        for (int i = 0; i < 4; i++) {
                c[i] = ((4 - i) * Sb[3 - i] / N - Sa[3 - i]) * tmp;
                tmp *= N;
        }
        for (int i = 0; i < 3; i++) {
                if (i >= n) break;
                const double Bi = screening[i];
                double d = 1. - Bi / N;
                d *= d;
                d *= d;
                a[i] = (a[i] - 4 * b[i] / (N - Bi)) / d;
                b[i] /= d;
        }
}

/* coulomb_transport_coefficients, order 0 only (pumas.c:7623-7683),
 * N = screening[n]. */
GPD double gp_coulomb_cs0(double mu, double S, int n_parameters,
    const double * screening, double N, const double * a, const double * b,
    const double * c)
{
        const int n = n_parameters - 1;
        double cs0 = 0.;
        for (int i = 0; i < 3; i++) {
                if (i >= n) break;
                const double alp = screening[i];
                const double r = mu / (mu + alp);
                const double L = gp_log(1. + mu / alp);
                const double I0 = r / alp;
                const double J0 = L;
                const double I1 = L - r;
                const double J1 = -alp * L;
                cs0 += a[i] * (J0 - S * J1) + b[i] * (I0 - S * I1);
        }
        const double r = mu / (mu + N);
        const double L = gp_log(1. + mu / N);
        const double I0 = r / N;
        const double J0 = L;
        const double I1 = L - r;
        const double J1 = -N * L;
        const double rn = 1. / (1. + mu / N);
        const double K0 = (1. - rn) * (1. + rn) / (2 * N * N);
        const double L0 =
            (1. - rn) * ((1. + rn) * (1. + rn) - rn) / (3 * N * N * N);
        const double K1 = I0 - N * K0;
        const double L1 = K0 - N * L0;
        cs0 += c[0] * (J0 - S * J1) + c[1] * (I0 - S * I1) +
            c[2] * (K0 - S * K1) + c[3] * (L0 - S * L1);
        return cs0;
}

/* coulomb_restricted_cs (pumas.c:7591-7609), N = screening[n]. */
GPD double gp_coulomb_restricted_cs(double mu, double fspin, int n_parameters,
    const double * screening, double N, const double * a, const double * b,
    const double * c)
{
        if ((mu >= 1.) || (mu >= 1E+06 * N))
                return 0.;
        const double cs0 =
            gp_coulomb_cs0(1., fspin, n_parameters, screening, N, a, b, c);
        const double cs = gp_coulomb_cs0(mu, fspin, n_parameters, screening,
            N, a, b, c);
        if (cs > cs0)
                return 0;
        else
                return cs0 - cs;
}

/* ------------------------------------------------------------------------ */
/* Numerical helpers and default DCS models.                                */
/* ------------------------------------------------------------------------ */

/* Gauss-Legendre nodes and weights on [0, 1], 9 and 12 points, as in
 * math_gauss_quad_coefficients (pumas.c:12463-12561). */
static __constant__ double gp_gl9_x[9] = {
        0.0159198802461870, 0.0819844463366821, 0.1933142836497048,
        0.3378732882980955, 0.5000000000000000, 0.6621267117019045,
        0.8066857163502952, 0.9180155536633179, 0.9840801197538130,
};
static __constant__ double gp_gl9_w[9] = {
        0.0406371941807872, 0.0903240803474287, 0.1303053482014677,
        0.1561735385200015, 0.1651196775006299, 0.1561735385200015,
        0.1303053482014677, 0.0903240803474287, 0.0406371941807872,
};
static __constant__ double gp_gl12_x[12] = {
        0.0092196828766404, 0.0479413718147625, 0.1150486629028477,
        0.2063410228566913, 0.3160842505009099, 0.4373832957442655,
        0.5626167042557344, 0.6839157494990901, 0.7936589771433087,
        0.8849513370971523, 0.9520586281852375, 0.9907803171233596,
};
static __constant__ double gp_gl12_w[12] = {
        0.0235876681932559, 0.0534696629976592, 0.0800391642716731,
        0.1015837133615330, 0.1167462682691774, 0.1245735229067014,
        0.1245735229067014, 0.1167462682691774, 0.1015837133615330,
        0.0800391642716731, 0.0534696629976592, 0.0235876681932559,
};

/* Chebyshev coefficients of CERNLIB RDILOG (C332), math_dilog
 * (pumas.c:12609-12673). */
static __constant__ double gp_dilog_c[20] = {
        0.42996693560813697, 0.40975987533077105, -0.01858843665014592,
        0.00145751084062268, -0.00014304184442340, 0.00001588415541880,
        -0.00000190784959387, 0.00000024195180854, -0.00000003193341274,
        0.00000000434545063, -0.00000000060578480, 0.00000000008612098,
        -0.00000000001244332, 0.00000000000182256, -0.00000000000027007,
        0.00000000000004042, -0.00000000000000610, 0.00000000000000093,
        -0.00000000000000014, 0.00000000000000002,
};

GPD double gp_sq(double x) { return x * x; }

/* math_dilog (pumas.c:12609-12673); pow(y, 2.) is exactly y * y. */
static __device__ double gp_dilog(double x)
{
        const double PI3 = GP_PI * GP_PI / 3.;
        const double PI6 = GP_PI * GP_PI / 6.;
        const double PI12 = GP_PI * GP_PI / 12.;
        if (x == 10) {
                return PI6;
        } else if ((x == -1.) || (1. - x == 0.)) {
                return -PI12;
        }
        double T = -x;
        double A, S, Y;
        if (T <= -2) {
                Y = -1. / (1. + T);
                S = 1.;
                A = -PI3 + 0.5 * (gp_sq(gp_log(-T)) - gp_sq(gp_log(1. + 1. / T)));
        } else if (T < -1.) {
                Y = -1. - T;
                S = -1.;
                A = gp_log(-T);
                A = -PI6 + A * (A + gp_log(1. + 1. / T));
        } else if (T <= -0.5) {
                Y = -(1. + T) / T;
                S = 1.;
                A = gp_log(-T);
                A = -PI6 + A * (-0.5 * A + gp_log(1. + T));
        } else if (T < 0.) {
                Y = -T / (1. + T);
                S = -1.;
                A = 0.5 * gp_sq(gp_log(1 + T));
        } else if (T <= 1.) {
                Y = T;
                S = 1.;
                A = 0.;
        } else {
                Y = 1. / T;
                S = -1.;
                A = PI6 + 0.5 * gp_sq(gp_log(T));
        }
        const double H = Y + Y - 1;
        const double ALFA = H + H;
        double B0 = 0., B1 = 0., B2 = 0.;
#pragma unroll
        for (int i = 19; i >= 0; i--) {
                B0 = gp_dilog_c[i] + ALFA * B1 - B2;
                B2 = B1;
                B1 = B0;
        }
        return -(S * (B0 - H * B2) + A);
}

#define GP_SSR_SQRTE 1.648721270700128
#define GP_SSR_ME 0.5109989461
#define GP_SSR_RE 2.8179403227E-13

/* dcs_bremsstrahlung_SSR (pumas.c:13915-14005), in m^2/GeV. */
static __device__ double gp_dcs_bremsstrahlung(const gp_tables & T,
    const gp_element & el, double K, double q)
{
        double m = T.mass;
        const double Z = el.Z;
        if ((Z <= 0) || (el.A <= 0) || (m <= 0) || (K <= 0) || (q <= 0))
                return 0.;
        if (q >= K + m * el.qmax_m_brems) return 0.;
        const double energy = (K + m) * 1E+03;
        const double v = q * 1E+03 / energy;
        m *= 1E+03;
        const double Z13 = el.z13_inv;
        const double rad_log = el.rad_log;
        const double rad_log_inel = (Z == 1.) ? 446. : 1429.;
        const double delta = m * m * v / (2. * energy * (1. - v));
        double phi1 = gp_log(rad_log * Z13 * (m / GP_SSR_ME) /
            (1. + rad_log * Z13 * T.k.exp_half * delta / GP_SSR_ME));
        double phi2 = gp_log(rad_log * Z13 * T.k.exp_m16 * (m / GP_SSR_ME) /
            (1. + rad_log * Z13 * T.k.exp_13 * delta / GP_SSR_ME));
        phi1 -= el.ssr_delta1 * (1. - 1. / Z);
        phi2 -= el.ssr_delta2 * (1. - 1. / Z);
        const double s_atomic_1 = gp_log(
            m / delta / (m * delta / (GP_SSR_ME * GP_SSR_ME) + GP_SSR_SQRTE));
        const double s_atomic_2 = gp_log(1. + GP_SSR_ME /
            (delta * rad_log_inel * Z13 * Z13 * GP_SSR_SQRTE));
        const double s_atomic =
            (4. / 3. * (1. - v) + v * v) * (s_atomic_1 - s_atomic_2);
        double s_rad;
        if (v < .0 || v > 1.) {
                s_rad = 0.;
        } else if (v < 0.02) {
                s_rad = -0.00349 + 148.84 * v + -987.531 * v * v;
        } else if (v >= 0.02 && v < 0.1) {
                s_rad = 0.1642 + 132.573 * v + -585.361 * v * v +
                    1407.77 * v * v * v;
        } else if (v >= 0.01 && v < 0.9) {
                s_rad = -2.8922 + -19.0156 * v + 57.698 * v * v;
                const double tmp = gp_log(1. - v);
                s_rad += -63.418 * v * gp_log(v) + 14.1166 * tmp +
                    1.84206 * tmp * tmp;
        } else {
                s_rad = 2134.19 + 581.823 * v + -2708.85 * v * v;
                const double tmp = gp_log(1. - v);
                s_rad += 4767.05 * v * gp_log(v) + 1.52918 * tmp +
                    0.361933 * tmp * tmp;
        }
        const double result =
            ((2. - 2. * v + v * v) * phi1 - 2. / 3. * (1. - v) * phi2) +
            1. / Z * s_atomic + 0.25 * GP_ALPHA_EM * phi1 * s_rad;
        if (result <= 0.) return 0.;
        const double aux = 2 * (GP_SSR_ME / m) * GP_SSR_RE * Z;
        return aux * aux * (GP_ALPHA_EM / q) * result * 1E-04;
}

/* dcs_pair_production_d2_SSR (pumas.c:14394-14544). */
static __device__ double gp_dcs_pair_d2(const gp_tables & T, const gp_element & el,
    double K, double q, double rho)
{
        double m = T.mass;
        const double Z = el.Z;
        if ((Z <= 0) || (el.A <= 0) || (m <= 0) || (K <= 0) || (q <= 0))
                return 0.;
        const double qmin = 4. * GP_ELECTRON_MASS;
        const double qmax = K + m * el.qmax_m_pair;
        if ((q < qmin) || (q > qmax)) return 0.;
        const double energy = (K + m) * 1E+03;
        const double v = q / (K + m);
        m *= 1E+03;
        const double rad_log = el.rad_log;
        const double const_prefactor = el.pair_pref;
        const double Z13 = el.zm13;
        const double d_n = el.dn;
        rho = 1 - rho;
        const double rho2 = rho * rho;
        double g1, g2;
        if (Z == 1.) {
                g1 = 4.4E-05;
                g2 = 4.8E-05;
        } else {
                g1 = 1.95E-05;
                g2 = 5.3E-05;
        }
        const double zeta1 =
            (0.073 * gp_log(energy / m / (1. + g1 * el.z23 * energy / m)) - 0.26);
        const double zeta2 =
            (0.058 * gp_log(energy / m / (1 + g2 / Z13 * energy / m)) - 0.14);
        double zeta;
        if ((zeta1 > 0.) && (zeta2 > 0.))
                zeta = zeta1 / zeta2;
        else
                zeta = 0.;
        const double beta = v * v / (2. * (1. - v));
        const double xi =
            gp_sq(m * v / (2. * GP_SSR_ME)) * (1. - rho2) / (1. - v);
        const double lxi = gp_log(1. + 1. / xi);
        const double Be = ((2. + rho2) * (1. + beta) + xi * (3. + rho2)) * lxi +
            (1. - rho2 - beta) / (1. + xi) - (3. + rho2);
        const double Ce2 = ((1. - rho2) * (1. + beta) + xi * (3. - rho2)) * lxi +
            2. * (1. - beta - rho2) / (1. + xi) - (3. - rho2);
        const double Ce1 = Be - Ce2;
        const double De = ((2. + rho2) * (1. + beta) + xi * (3. + rho2)) *
                gp_dilog(1. / (1. + xi)) -
            (2. + rho2) * xi * lxi - (xi + rho2 + beta) / (1. + xi);
        const double sxi = sqrt(1. + xi);
        const double ev = energy * v * (1. - rho2);
        double Le1, Le2;
        if (De / Be > 0.) {
                const double tmp = De / Be;
                const double Xe = (tmp < 100) ? gp_exp(-tmp) : 0.;
                Le1 = gp_log(rad_log * Z13 * sxi /
                          (Xe + 2. * GP_SSR_ME * T.k.exp_half * rad_log * Z13 *
                                  (1. + xi) / ev)) - tmp -
                    0.5 * gp_log(Xe + el.pair_medn2 * (1. + xi));
                Le2 = gp_log(rad_log * Z13 * T.k.exp_m16 * sxi /
                          (Xe + 2. * GP_SSR_ME * T.k.exp_13 * rad_log * Z13 *
                                  (1. + xi) / ev)) - tmp -
                    0.5 * gp_log(Xe + el.pair_medn2 * T.k.exp_m13 * (1. + xi));
        } else {
                const double tmp = De / Be;
                const double Xe_inv = (tmp > -100) ? gp_exp(De / Be) : 0;
                Le1 = gp_log(rad_log * Z13 * sxi /
                          (1. + Xe_inv * 2. * GP_SSR_ME * T.k.exp_half *
                                    rad_log * Z13 * (1. + xi) / ev)) -
                    0.5 * De / Be -
                    0.5 * gp_log(1. + Xe_inv * el.pair_medn2 * (1. + xi));
                Le2 = gp_log(rad_log * Z13 * T.k.exp_m16 * sxi /
                          (1. + Xe_inv * 2. * GP_SSR_ME * T.k.exp_13 *
                                    rad_log * Z13 * (1. + xi) / ev)) -
                    0.5 * De / Be -
                    0.5 * gp_log(1. + Xe_inv * el.pair_medn2 * T.k.exp_m13 *
                                       (1. + xi));
        }
        double diagram_e = const_prefactor * (Z + zeta) * (1. - v) / v *
            (Ce1 * Le1 + Ce2 * Le2);
        if (diagram_e < 0.) diagram_e = 0.;

        const double lxi1 = gp_log(1. + xi);
        const double Bm = ((1. + rho2) * (1. + (3. * beta) / 2) -
                              1. / xi * (1. + 2. * beta) * (1. - rho2)) * lxi1 +
            xi * (1. - rho2 - beta) / (1. + xi) +
            (1. + 2. * beta) * (1. - rho2);
        const double Cm2 =
            ((1. - beta) * (1. - rho2) - xi * (1. + rho2)) * lxi1 / xi -
            2. * (1. - beta - rho2) / (1. + xi) + 1. - beta -
            (1. + beta) * rho2;
        const double Cm1 = Bm - Cm2;
        const double Dm = ((1. + rho2) * (1. + (3. * beta) / 2.) -
                              1. / xi * (1. + 2. * beta) * (1. - rho2)) *
                gp_dilog(xi / (1. + xi)) +
            (1. + (3. * beta) / 2.) * (1. - rho2) / xi * lxi1 +
            (1. - rho2 - beta / 2. * (1. + rho2) +
                (1. - rho2) / (2. * xi) * beta) * xi / (1. + xi);
        double Lm1, Lm2;
        if (Dm / Bm > 0.) {
                const double tmp = Dm / Bm;
                const double Xm = (tmp < 100) ? gp_exp(-tmp) : 0.;
                Lm1 = gp_log(m / GP_SSR_ME * rad_log * Z13 / d_n /
                          (Xm + 2. * GP_SSR_ME * T.k.exp_half * rad_log * Z13 *
                                  (1. + xi) / ev)) - tmp;
                Lm2 = gp_log(m / GP_SSR_ME * rad_log * Z13 / d_n /
                          (Xm + 2. * GP_SSR_ME * T.k.exp_13 * rad_log * Z13 *
                                  (1. + xi) / ev)) - tmp;
        } else {
                const double tmp = Dm / Bm;
                const double Xmv = (tmp > -100) ? gp_exp(tmp) : 0.;
                Lm1 = gp_log(m / GP_SSR_ME * rad_log * Z13 / d_n /
                    (1. + 2. * GP_SSR_ME * T.k.exp_half * rad_log * Z13 *
                            (1. + xi) / ev * Xmv));
                Lm2 = gp_log(m / GP_SSR_ME * rad_log * Z13 / d_n /
                    (1. + 2. * GP_SSR_ME * T.k.exp_13 * rad_log * Z13 *
                            (1. + xi) / ev * Xmv));
        }
        double diagram_mu = const_prefactor * (Z + zeta) * (1. - v) / v *
            T.k.pair_me_m2 * (Cm1 * Lm1 + Cm2 * Lm2);
        if (diagram_mu < 0.) diagram_mu = 0.;
        return (diagram_e + diagram_mu) * 1E-01 / energy;
}

/* dcs_pair_production_SSR (pumas.c:14560-14604). */
static __device__ double gp_dcs_pair_production(const gp_tables & T,
    const gp_element & el, double K, double q)
{
        const double mass = T.mass;
        if ((el.Z <= 0) || (el.A <= 0) || (mass <= 0) || (K <= 0) || (q <= 0))
                return 0.;
        if (q <= 4. * GP_ELECTRON_MASS) return 0.;
        if (q >= K + mass * el.qmax_m_pair) return 0.;
        const double gamma = 1. + K / mass;
        const double x0 = 1. - 4. * GP_ELECTRON_MASS / q;
        const double x1 = 1. - 6. / (gamma * (gamma - q / mass));
        double rmax;
        if ((x0 > 0) && (x1 > 0))
                rmax = sqrt(x0) * x1;
        else
                return 0.;
        const double ri = 1. - rmax;
        if ((ri <= 0.) || (ri >= 1.)) return 0.;
        const double tmin = gp_log(ri);
        double I = 0.;
        for (int i = 0; i < 12; i++) {
                const double rho = gp_exp(gp_gl12_x[i] * tmin);
                I -= gp_dcs_pair_d2(T, el, K, q, rho) * rho * gp_gl12_w[i] *
                    tmin;
        }
        return (I < 0) ? 0. : I;
}

/* dcs_photonuclear_f2p_ALLM97 (pumas.c:14626-14673). */
GPD double gp_f2p_allm97(const gp_tables & T, double x, double Q2)
{
        const double m02 = 0.31985;
        const double mP2 = 49.457;
        const double mR2 = 0.15052;
        const double Q02 = 0.52544;
        const double Lambda2 = 0.06527;
        const double M = 0.5 * (GP_PROTON_MASS + GP_NEUTRON_MASS);
        const double M2 = M * M;
        const double W2 = M2 + Q2 * (1.0 / x - 1.0);
        const double t = gp_log(gp_log((Q2 + Q02) / Lambda2) / T.k.allm_lq0);
        const double xP = (Q2 + mP2) / (Q2 + mP2 + W2 - M2);
        const double xR = (Q2 + mR2) / (Q2 + mR2 + W2 - M2);
        /* The six powers of t share one logarithm: t^c = exp(c ln t), exact
         * to a few ulps (t = 0 gives exp(-inf) = 0 as pow). */
        const double lt = gp_log(t);
        const double cP = 0.28067 +
            (0.28067 - 0.22291) * (1.0 / (1.0 + gp_exp(2.1979 * lt)) - 1.0);
        const double aP = -0.0808 +
            (-0.0808 - -0.44812) * (1.0 / (1.0 + gp_exp(1.1709 * lt)) - 1.0);
        const double bP = 0.36292 + 1.8917 * gp_exp(1.8439 * lt);
        const double cR = 0.80107 + 0.97307 * gp_exp(3.4942 * lt);
        const double aR = 0.58400 + 0.37888 * gp_exp(2.6063 * lt);
        const double bR = 0.01147 + 3.7582 * gp_exp(0.49338 * lt);
        const double l1x = gp_log(1 - x);
        const double F2P = cP * gp_exp(aP * gp_log(xP) + bP * l1x);
        const double F2R = cR * gp_exp(aR * gp_log(xR) + bR * l1x);
        return Q2 / (Q2 + m02) * (F2P + F2R);
}

/* dcs_photonuclear_d2_DRSS (pumas.c:14923-14943) with the shadowing and F2
 * of pumas.c:14688-14721. */
static __device__ double gp_photonuclear_d2(const gp_tables & T,
    const gp_element & el, double K, double q, double Q2)
{
        const double ml = T.mass;
        const double cf = 4 * GP_PI * GP_ALPHA_EM * GP_ALPHA_EM * GP_HBAR_C *
            GP_HBAR_C;
        const double M = 0.5 * (GP_PROTON_MASS + GP_NEUTRON_MASS);
        const double E = K + ml;
        const double y = q / E;
        const double x = 0.5 * Q2 / (M * q);
        const double F2p = gp_f2p_allm97(T, x, Q2);
        const double Z = el.Z, A = el.A;
        double shadowing;
        if (Z == 1.)
                shadowing = 1.;
        else if (x < 0.0014)
                shadowing = el.shadow_low;
        else if (x < 0.04)
                shadowing = gp_exp((0.069 * log10(x) + 0.097) * el.log_A);
        else
                shadowing = 1.;
        const double F2A = F2p * shadowing *
            (Z + (A - Z) * (1.0 + x * (-1.85 + x * (2.45 + x * (-2.35 + x)))));
        const double R = 0.;
        const double dds = (1 - y +
                               0.5 * (1 - 2 * ml * ml / Q2) *
                                   (y * y + Q2 / (E * E)) / (1 + R)) /
                (Q2 * Q2) -
            0.25 / (E * E * Q2);
        return cf * F2A * dds / q;
}

/* The doubly differential cross section of the photonuclear polar angle
 * sampler: the BM model's for BM, else DRSS's (dcs_photonuclear_ddcs,
 * pumas.c:15159-15170). */
GPD double gp_photonuclear_ddcs(const gp_tables & T, const gp_element & el,
    double K, double q, double Q2)
{
        if (T.model_photo == 2)
                return gpm_photonuclear_d2_BM(el.Z, el.A, T.mass, K, q, Q2);
        return gp_photonuclear_d2(T, el, K, q, Q2);
}

/* dcs_photonuclear_DRSS (pumas.c:15002-15083, mode 0). */
static __device__ double gp_dcs_photonuclear(const gp_tables & T,
    const gp_element & el, double K, double q)
{
        const double ml = T.mass;
        if ((el.Z <= 0) || (el.A <= 0) || (ml <= 0) || (K <= 0)) return 0.;
        const double M = 0.5 * (GP_NEUTRON_MASS + GP_PROTON_MASS);
        const double mpi = GP_PION_MASS;
        if ((q <= mpi + 0.5 * mpi * mpi / M) ||
            (q >= K + ml - 0.5 * (M + ml * ml / M)))
                return 0.;
        const double E = K + ml;
        const double ml2 = ml * ml;
        const double Q2min = ml2 * (q * q - 0.5 * ml2) / (E * (E - q));
        const double Q2max = 2.0 * M * (q - mpi) - mpi * mpi;
        if ((Q2max < Q2min) | (Q2min < 0)) return 0.;
        const double xmin = gp_log(Q2min);
        const double xmax = gp_log(Q2max);
        const double dx = xmax - xmin;
        double ds = 0.;
        for (int i = 0; i < 9; i++) {
                const double Q2 = gp_exp(xmin + dx * gp_gl9_x[i]);
                const double w = gp_gl9_w[i] * (dx * Q2);
                const double tmp = gp_photonuclear_d2(T, el, K, q, Q2);
                if (tmp <= 0.) continue;
                ds += tmp * w;
        }
        return (ds < 0.) ? 0. : ds;
}

GPD void gp_photonuclear_range(
    double m, double K, double & qmin, double & qmax)
{
        const double M = 0.5 * (GP_NEUTRON_MASS + GP_PROTON_MASS);
        const double mpi = GP_PION_MASS;
        qmin = mpi + 0.5 * mpi * mpi / M;
        qmax = K + m - 0.5 * (M + m * m / M);
}

/* pumas_electronic_dcs (pumas.c:11082-11101). */
GPD double gp_electronic_dcs(double Z, double I, double m, double K, double q)
{
        const double P2 = K * (K + 2. * m);
        const double E = K + m;
        const double Wmax = 2. * GP_ELECTRON_MASS * P2 /
            (m * m + GP_ELECTRON_MASS * (GP_ELECTRON_MASS + 2. * E));
        if (q > Wmax) return 0.;
        const double Wmin = (13.6 / 19.2) * I;
        if (q <= Wmin) return 0.;
        const double E2 = E * E;
        const double beta2 = P2 / E2;
        const double a0 = 0.5 / E2;
        const double a1 = beta2 / Wmax;
        return 2 * GP_PI * GP_ELECTRON_MASS * GP_ELECTRON_RADIUS *
            GP_ELECTRON_RADIUS * Z * (a0 + 1. / q * (1 / q - a1)) / beta2;
}

/* Process DCS wrappers (pumas.c:11003-11122), in m^2/kg. */
static __device__ double gp_dcs_process(const gp_tables & T, int process,
    const gp_element & el, double K, double q)
{
        const double m = T.mass;
        if (process == 0) {
                /* The dump's model (struct pumas_physics_settings). */
                const double d = (T.model_brems == 0) ?
                    gp_dcs_bremsstrahlung(T, el, K, q) :
                    (T.model_brems == 1) ?
                    gpm_bremsstrahlung_KKP(el.Z, el.A, m, K, q, el.rad_log) :
                    gpm_bremsstrahlung_ABB(el.Z, el.A, m, K, q);
                return d * 1E+03 * GP_AVOGADRO * (m + K) / el.A;
        } else if (process == 1) {
                const double d = (T.model_pair == 0) ?
                    gp_dcs_pair_production(T, el, K, q) :
                    gpm_pair_production_KKP(el.Z, el.A, m, K, q, el.rad_log,
                        gp_gl12_x, gp_gl12_w);
                return d * 1E+03 * GP_AVOGADRO * (m + K) / el.A;
        } else if (process == 2) {
                double qmin, qmax;
                gp_photonuclear_range(m, K, qmin, qmax);
                if ((q < qmin) || (q > qmax)) return 0.;
                const double d = (T.model_photo == 0) ?
                    gp_dcs_photonuclear(T, el, K, q) :
                    (T.model_photo == 1) ?
                    gpm_photonuclear_BBKS(el.Z, el.A, m, K, q) :
                    gpm_photonuclear_BM(el.Z, el.A, m, K, q, gp_gl9_x,
                        gp_gl9_w);
                return d * 1E+03 * GP_AVOGADRO * (m + K) / el.A;
        } else {
                return gp_electronic_dcs(el.Z, el.I, m, K, q) * (m + K) *
                    GP_AVOGADRO / (el.A * 1E-03);
        }
}

/* Single precision log and exp with the C library's results on the DCS
 * domains (gp_libmf.cuh). */
GPD float gp_logf(float x) { return gp_libm_logf(x); }
GPD float gp_expf(float x) { return gp_libm_expf(x); }

/* dcs_evaluate (pumas.c:11243-11347). */
static __device__ double gp_dcs_evaluate(const gp_tables & T, int process,
    const gp_element & el, double K, double q)
{
        const double wj = K / (K + T.mass);
        if (process == 3) return gp_dcs_process(T, 3, el, K, q) * wj;
        double qlow = 0;
        if (process == 2) {
                double qmin, qmax;
                gp_photonuclear_range(T.mass, K, qmin, qmax);
                if ((q < qmin) || (q > qmax))
                        return 0.;
                else
                        qlow = 2 * qmin;
        } else {
                double qmin = 4. * GP_ELECTRON_MASS;
                const double qmax = K + T.mass * el.qmax_m_pair;
                if (process == 1)
                        qlow = 4 * qmin;
                else
                        qmin = 0.;
                if ((q < qmin) || (q > qmax)) return 0.;
        }
        if (q < qlow) return gp_dcs_process(T, process, el, K, q) * wj;

        const int nx = T.n_table_dcs;
        const float xmin = __ldg(T.DCS_x);
        const float xmax = __ldg(T.DCS_x + nx - 1);
        const float x = gp_logf((float)(q / K));
        if ((x < xmin) || (x >= xmax))
                return gp_dcs_process(T, process, el, K, q) * wj;
        int ix = 0, tmpi = nx - 1;
        do {
                const int i3 = (ix + tmpi) >> 1;
                if (x >= __ldg(T.DCS_x + i3))
                        ix = i3;
                else
                        tmpi = i3;
        } while (tmpi - ix >= 2);
        if ((ix < 0) || (ix >= nx - 1))
                return gp_dcs_process(T, process, el, K, q) * wj;

        float p00, p01, m00, m01, p10, p11, m10, m11, h0, h1;
        const int imax = T.n_energies - 1;
        const double Kmax = __ldg(T.K + imax);
        const long stride = (long)nx * 2;
        const float * base = T.DCS +
            stride * ((long)(process * T.n_elements + el.index) * T.n_energies);
        int i0 = 0;
        if ((K >= Kmax) || ((i0 = gp_index(T, GP_LUT_K, T.K, K)) >= imax)) {
                const float * data = base + stride * imax;
                p00 = p10 = __ldg(data + 2 * ix);
                m00 = m10 = __ldg(data + 2 * ix + 1);
                p01 = p11 = __ldg(data + 2 * ix + 2);
                m01 = m11 = __ldg(data + 2 * ix + 3);
                h0 = 1.f;
                h1 = 0.f;
        } else {
                const float * data = base + stride * i0;
                p00 = __ldg(data + 2 * ix);
                m00 = __ldg(data + 2 * ix + 1);
                p01 = __ldg(data + 2 * ix + 2);
                m01 = __ldg(data + 2 * ix + 3);
                data += 2 * nx;
                p10 = __ldg(data + 2 * ix);
                m10 = __ldg(data + 2 * ix + 1);
                p11 = __ldg(data + 2 * ix + 2);
                m11 = __ldg(data + 2 * ix + 3);
                const float K0 = (float)__ldg(T.K + i0);
                const float K1 = (float)__ldg(T.K + i0 + 1);
                h1 = __fdiv_rn(gp_logf(__fdiv_rn((float)K, K0)),
                    gp_logf(__fdiv_rn(K1, K0)));
                h0 = __fsub_rn(1.f, h1);
        }
        if (((p00 == 0.f) && (m00 == 0.f)) || ((p01 == 0.f) && (m01 == 0.f)) ||
            ((p10 == 0.f) && (m10 == 0.f)) || ((p11 == 0.f) && (m11 == 0.f)))
                return gp_dcs_process(T, process, el, K, q) * wj;

        /* Single precision interpolation, without fused multiply-adds as
         * the reference's SSE evaluation. */
        const float x0 = __ldg(T.DCS_x + ix);
        const float x1 = __ldg(T.DCS_x + ix + 1);
        const float dx = __fsub_rn(x1, x0);
        m00 = __fmul_rn(m00, dx);
        m01 = __fmul_rn(m01, dx);
        const float t = __fdiv_rn(__fsub_rn(x, x0), dx);
        const float d0 = __fsub_rn(p00, p01);
        const float c02 = __fsub_rn(__fsub_rn(__fmul_rn(-3.f, d0),
            __fmul_rn(2.f, m00)), m01);
        const float c03 = __fadd_rn(__fadd_rn(__fmul_rn(2.f, d0), m00), m01);
        float r = __fmul_rn(gp_expf(__fadd_rn(p00, __fmul_rn(t, __fadd_rn(m00,
            __fmul_rn(t, __fadd_rn(c02, __fmul_rn(t, c03))))))), h0);
        if (h1 > 0.f) {
                m10 = __fmul_rn(m10, dx);
                m11 = __fmul_rn(m11, dx);
                const float d1 = __fsub_rn(p10, p11);
                const float c12 = __fsub_rn(__fsub_rn(__fmul_rn(-3.f, d1),
                    __fmul_rn(2.f, m10)), m11);
                const float c13 =
                    __fadd_rn(__fadd_rn(__fmul_rn(2.f, d1), m10), m11);
                r = __fadd_rn(r, __fmul_rn(gp_expf(__fadd_rn(p10,
                    __fmul_rn(t, __fadd_rn(m10, __fmul_rn(t, __fadd_rn(c12,
                    __fmul_rn(t, c13))))))), h1));
        }
        return r * wj;
}

/* ------------------------------------------------------------------------ */
/* Event context helpers.                                                   */
/* ------------------------------------------------------------------------ */

/* Medium of a geometry region: material and density (transport_set_locals,
 * pumas.c:5528-5552, for a uniform density override). */
GPD int gp_medium_material(const gpumas_geometry & g, int medium)
{
        return __ldg(&g.media[medium].material);
}

GPD double gp_medium_density(
    const gp_tables & T, const gpumas_geometry & g, int medium)
{
        const double d = __ldg(&g.media[medium].density);
        return (d > 0.) ? d : __ldg(T.material_density +
                                  __ldg(&g.media[medium].material));
}

/* Local properties of the current medium on a geometry with locals
 * (struct medium_locals, pumas.c:396-403): its field, density and step
 * limit. Without locals the transport functions get a NULL gp_loc and
 * compile without this code. */
struct gp_loc {
        const gpumas_geometry * g;
        double magnet[3];
        double density;  /* density at the end of the last step */
        double step_max; /* step_max_locals: size x accuracy, 0: uniform */
        int magnetized;
};

/* transport_set_locals (pumas.c:5528-5552) for medium `medium` of a
 * geometry with locals, at the event's position and direction: sets the
 * density and the field and returns the step limit (0: uniform). */
GPD double gp_set_locals(const gp_tables & T, const gp_config & cfg,
    const gp_event & e, int medium, double & density, gp_loc & loc)
{
        const gpumas_geometry & g = *loc.g;
        const gpumas_locals * l = g.locals + medium;
        double size = 0.;
        if (__ldg(&l->model) == GPUMAS_DENSITY_EXPONENTIAL) {
                gpumas_locals lc;
                lc.axis[0] = __ldg(l->axis), lc.axis[1] = __ldg(l->axis + 1);
                lc.axis[2] = __ldg(l->axis + 2);
                lc.h0 = __ldg(&l->h0), lc.lambda = __ldg(&l->lambda);
                lc.eps = __ldg(&l->eps);
                density = GP_MUL(__ldg(&l->rho0),
                    gp_exp(gpumas_locals_exponent(&lc, e.pos)));
                size = gpumas_locals_size(&lc, e.dir);
        } else {
                density = __ldg(&g.media[medium].density);
        }
        if (density <= 0.)
                density = __ldg(T.material_density +
                    __ldg(&g.media[medium].material));
        loc.magnet[0] = __ldg(l->magnet);
        loc.magnet[1] = __ldg(l->magnet + 1);
        loc.magnet[2] = __ldg(l->magnet + 2);
        loc.magnetized = ((loc.magnet[0] != 0.) || (loc.magnet[1] != 0.) ||
                             (loc.magnet[2] != 0.)) ? 1 : 0;
        return GP_MUL(size, cfg.accuracy);
}

/* Larmor radius and deflection direction (u x B) / p of a step end point
 * (pumas.c:6352-6378, 6850-6872): returns 0 without transverse field. */
GPD double gp_larmor(const double * u, const double * B, double p,
    double * uT)
{
        uT[0] = GP_SUB(GP_MUL(u[1], B[2]), GP_MUL(u[2], B[1]));
        uT[1] = GP_SUB(GP_MUL(u[2], B[0]), GP_MUL(u[0], B[2]));
        uT[2] = GP_SUB(GP_MUL(u[0], B[1]), GP_MUL(u[1], B[0]));
        const double BT = sqrt(GP_ADD(GP_ADD(GP_MUL(uT[0], uT[0]),
            GP_MUL(uT[1], uT[1])), GP_MUL(uT[2], uT[2])));
        if (BT == 0.) return 0.;
        const double pinv = 1. / p;
        uT[0] = GP_MUL(uT[0], pinv);
        uT[1] = GP_MUL(uT[1], pinv);
        uT[2] = GP_MUL(uT[2], pinv);
        return p / GP_MUL(BT, GP_LARMOR_FACTOR);
}

GPD int gp_locate(const gpumas_geometry & g, const gp_event & e)
{
        return gpumas_geometry_locate(&g, e.pos);
}

GPD double gp_step_proposal(const gp_config & cfg, const gpumas_geometry & g,
    gp_event & e, int medium)
{
        const double sgn = (cfg.direction == GPUMAS_MODE_FORWARD) ? 1. : -1.;
        const double u[3] = { sgn * e.dir[0], sgn * e.dir[1], sgn * e.dir[2] };
        e.steps++;
        return gpumas_geometry_step(&g, e.pos, u, medium);
}

/* step_randn (pumas.c:7016-7029): Box-Muller pairs cached per event. */
GPD double gp_randn(gp_event & e)
{
        e.randn_done = !e.randn_done;
        if (!e.randn_done) return e.randn_next;
        const double r = sqrt(-2. * gp_log(gp_random(e)));
        const double phi = GP_MUL(2. * GP_PI, gp_random(e));
        double s, c;
        sincos(phi, &s, &c);
        e.randn_next = GP_MUL(r, c);
        return GP_MUL(r, s);
}

/* step_rotate_direction (pumas.c:7042-7095), every product and sum
 * rounded on its own as in the reference's C code. */
GPD double gp_rnorm2(double a, double b)
{
        return __drcp_rn(sqrt(GP_ADD(GP_MUL(a, a), GP_MUL(b, b))));
}

GPD double gp_cross(double a, double b, double c, double d)
{
        return GP_SUB(GP_MUL(a, b), GP_MUL(c, d));
}

static __device__ __forceinline__ void gp_rotate(gp_event & e, double mu)
{
        double * const direction = e.dir;
        const double cos_theta = GP_SUB(1., GP_MUL(2., mu));
        const double stsq = GP_MUL(GP_MUL(4., mu), GP_SUB(1., mu));
        if (stsq <= 0.) return;
        const double st = sqrt(stsq);
        double u0x = 0., u0y = 0., u0z = 0.;
        const double d0 = direction[0], d1 = direction[1], d2 = direction[2];
        const double a0 = fabs(d0);
        const double a1 = fabs(d1);
        const double a2 = fabs(d2);
        if (a0 > a1) {
                if (a0 > a2) {
                        const double nrm = gp_rnorm2(d0, d2);
                        u0x = GP_MUL(-d2, nrm), u0z = GP_MUL(d0, nrm);
                } else {
                        const double nrm = gp_rnorm2(d1, d2);
                        u0y = GP_MUL(d2, nrm), u0z = GP_MUL(-d1, nrm);
                }
        } else {
                if (a1 > a2) {
                        const double nrm = gp_rnorm2(d0, d1);
                        u0x = GP_MUL(d1, nrm), u0y = GP_MUL(-d0, nrm);
                } else {
                        const double nrm = gp_rnorm2(d1, d2);
                        u0y = GP_MUL(d2, nrm), u0z = GP_MUL(-d1, nrm);
                }
        }
        const double u1x = gp_cross(u0y, d2, u0z, d1);
        const double u1y = gp_cross(u0z, d0, u0x, d2);
        const double u1z = gp_cross(u0x, d1, u0y, d0);
        /* phi = pi (1 - 2 u), 1 - 2 u being exact. */
        const double phi = GP_MUL(GP_PI, 1. - 2. * gp_random(e));
        double sp, cp;
        sincos(phi, &sp, &cp);
        direction[0] = GP_ADD(GP_MUL(cos_theta, d0),
            GP_MUL(st, GP_ADD(GP_MUL(cp, u0x), GP_MUL(sp, u1x))));
        direction[1] = GP_ADD(GP_MUL(cos_theta, d1),
            GP_MUL(st, GP_ADD(GP_MUL(cp, u0y), GP_MUL(sp, u1y))));
        direction[2] = GP_ADD(GP_MUL(cos_theta, d2),
            GP_MUL(st, GP_ADD(GP_MUL(cp, u0z), GP_MUL(sp, u1z))));
}

/* ------------------------------------------------------------------------ */
/* Polar angles of DELs (pumas.c:11736-11976).                              */
/* ------------------------------------------------------------------------ */

/* polar_bremsstrahlung (pumas.c:11759-11830), also for pair production. */
static __device__ __forceinline__ double gp_polar_bremsstrahlung(const gp_tables & T, gp_event & e,
    const gp_element & el, double ki, double kf)
{
        const double m = T.mass;
        const double E = ki + m;
        const double nu = ki - kf;
        const double y = nu / E;
        const double tmp = 0.5 * m * nu / (E * (E - nu));
        const double mu0 = tmp * tmp;
        const double c1 = (2 * (1. - y) + y * y) * mu0;
        const double c2 = 4 * (1. - y) * mu0 * mu0;
        const double muni = el.muni;
        const double muc = sqrt(mu0) - mu0;
        if (muc < 0) return 0;
        double x0;
        {
                const double q = muni;
                const double r = mu0;
                const double qr = q * r;
                x0 = (1. + 2 * qr) * gp_log((1. + qr) / (r + qr)) -
                    (1. - r) * (1 + 2 * q) / (1 + q);
        }
        for (int i = 0; i < 100; i++) {
                const double r0 = gp_random(e);
                const double r1 = gp_random(e);
                const double mu = r0 * mu0 / (mu0 + 1. - r0);
                const double mus = mu0 + mu;
                const double mu2 = mus * mus;
                const double d1 = 1 / mu2;
                const double d2 = d1 * d1;
                const double score = r1 * c1 * d1;
                double pdf = c1 * d1 - mu * c2 * d2;
                if (score > pdf) continue;
                const double l2 = mu2 / (mu0 * mu0);
                const double q = muni * l2;
                const double r = mu0 * l2;
                const double qr = q * r;
                if (qr > 1E+05) continue;
                const double x = (1. + 2 * qr) * gp_log((1. + qr) / (r + qr)) -
                    (1. - r) * (1 + 2 * q) / (1 + q);
                pdf *= x / x0;
                if (score <= pdf) return mu;
        }
        return 0.;
}

/* Objective of the photonuclear polar sampling (pumas.c:11855-11862). */
GPD double gp_polar_objective(const gp_tables & T, const gp_element & el,
    double K, double q, double lnQ2)
{
        const double Q2 = gp_exp(lnQ2);
        return -gp_photonuclear_ddcs(T, el, K, q, Q2) * Q2;
}

/* math_find_minimum_brent (pumas.c:12233-12325); as in the reference the
 * upper bracket of the search is the initial minimiser xb. */
static __device__ int gp_find_minimum_brent(const gp_tables & T,
    const gp_element & el, double K, double q, double xa, double xb,
    double xc, double fb, double tol, int max_iter, double & xopt,
    double & fopt)
{
        const double EPS = 1E-15;
        const double GOLD = 0.3819660;
        tol *= fabs(xc - xa);
        double x = xb, w = xb, v = xb;
        double fw = fb, fv = fb, fx = fb;
        double d = 0., ee = 0.;
        int i;
        for (i = 0; i < max_iter; i++) {
                const double xm = 0.5 * (xa + xb);
                const double tol1 = tol * fabs(x) + EPS;
                const double tol2 = 2 * tol1;
                if (fabs(x - xm) <= (tol2 - 0.5 * (xb - xa))) break;
                if (fabs(ee) > tol1) {
                        const double r = (x - w) * (fx - fv);
                        double qq = (x - v) * (fx - fw);
                        double p = (x - v) * qq - (x - w) * r;
                        qq = 2. * (qq - r);
                        if (qq > 0.) p = -p;
                        qq = fabs(qq);
                        const double etemp = ee;
                        ee = d;
                        if (fabs(p) >= fabs(0.5 * qq * etemp) ||
                            (p <= qq * (xa - x)) || (p >= qq * (xb - x))) {
                                ee = (x >= xm) ? xa - x : xb - x;
                                d = GOLD * ee;
                        } else {
                                d = p / qq;
                                const double u = x + d;
                                if ((u - xa < tol2) || (xb - u < tol2))
                                        d = ((xm - x) >= 0.0) ? fabs(tol1) :
                                                                -fabs(tol1);
                        }
                } else {
                        ee = (x >= xm) ? xa - x : xb - x;
                        d = GOLD * ee;
                }
                const double u = (fabs(d) >= tol1) ? x + d :
                    x + ((d >= 0.0) ? fabs(tol1) : -fabs(tol1));
                const double fu = gp_polar_objective(T, el, K, q, u);
                if (fu <= fx) {
                        if (u >= x)
                                xa = x;
                        else
                                xb = x;
                        v = w, w = x, x = u;
                        fv = fw, fw = fx, fx = fu;
                } else {
                        if (u < x)
                                xa = u;
                        else
                                xb = u;
                        if ((fu <= fw) || (w == x)) {
                                v = w;
                                w = u;
                                fv = fw;
                                fw = fu;
                        } else if ((fu <= fv) || (v == x) || (v == w)) {
                                v = u;
                                fv = fu;
                        }
                }
        }
        xopt = x;
        fopt = fx;
        return (i < max_iter) ? i : -1;
}

/* math_find_minimum with Brent refinement (pumas.c:12105-12206). */
static __device__ int gp_find_minimum(const gp_tables & T, const gp_element & el,
    double K, double q, double xa, double xc, double tol, int max_iter,
    double & xopt, double & fopt)
{
        double fa = gp_polar_objective(T, el, K, q, xa);
        double fc = gp_polar_objective(T, el, K, q, xc);
        const double atol = tol * fabs(xc - xa);
        double xb = 0, fb = 0;
        int i;
        for (i = 0; i < max_iter; i++) {
                xb = 0.5 * (xa + xc);
                fb = gp_polar_objective(T, el, K, q, xb);
                if ((fb < fa) && (fb < fc)) break;
                if (fabs(xc - xa) <= atol) {
                        xopt = xb;
                        fopt = fb;
                        return i;
                }
                if (fb < fc) {
                        xc = xb;
                        fc = fb;
                } else {
                        xa = xb;
                        fa = fb;
                }
        }
        if (i == max_iter) {
                if (fa < fb) {
                        fb = fa;
                        xb = xa;
                } else if (fc < fb) {
                        fb = fc;
                        xb = xc;
                }
                xopt = xb;
                fopt = fb;
                return -1;
        }
        const int status = gp_find_minimum_brent(
            T, el, K, q, xa, xb, xc, fb, tol, max_iter - i, xopt, fopt);
        return (status < 0) ? -2 : status + i;
}

/* polar_photonuclear (pumas.c:11874-11950). */
static __device__ __forceinline__ double gp_polar_photonuclear(const gp_tables & T, gp_event & e,
    const gp_element & el, double ki, double kf)
{
        const double M = 0.5 * (GP_PROTON_MASS + GP_NEUTRON_MASS);
        const double q = ki - kf;
        const double ml = T.mass;
        const double E = ki + ml;
        const double ml2 = ml * ml;
        const double Q2min = ml2 * (q * q - 0.5 * ml2) / (E * (E - q));
        const double Q2max =
            2.0 * M * (q - GP_PION_MASS) - GP_PION_MASS * GP_PION_MASS;
        if ((Q2max < Q2min) | (Q2min < 0)) return 0.;
        double fopt = 0., xopt = 0.;
        const double lnQ2min = gp_log(Q2min);
        const double lnQ2max = gp_log(Q2max);
        const int status = gp_find_minimum(
            T, el, ki, q, lnQ2min, lnQ2max, 1E-06, 100, xopt, fopt);
        fopt = -fopt;
        if (status == -2) return 0.;
        const double x = gp_exp(xopt) / (2 * q * M);
        const double lne = 0.1;
        if ((x <= 0.04) && (xopt + lne < lnQ2max)) {
                double f2, x2;
                const int status2 = gp_find_minimum(
                    T, el, ki, q, xopt + lne, lnQ2max, 1E-06, 100, x2, f2);
                if (status2 >= 0) {
                        f2 = -f2;
                        if (f2 > fopt) {
                                xopt = x2;
                                fopt = f2;
                        }
                }
        }
        const double rQ2 = lnQ2max - lnQ2min;
        double Q2 = 0.;
        int i;
        for (i = 0; i < 100; i++) {
                const double u = gp_random(e);
                Q2 = Q2min * gp_exp(rQ2 * u);
                const double r = gp_photonuclear_ddcs(T, el, ki, q, Q2) * Q2;
                if (gp_random(e) * fopt <= r) break;
        }
        if (i == 100) return 0.;
        const double p = sqrt(ki * (ki + 2 * ml));
        const double E1 = E - q;
        const double eps = ml / E1;
        const double p1 = E1 * sqrt((1. + eps) * (1. - eps));
        const double p2 = p * p1;
        double tmp = GP_SUB(GP_ADD(p2, GP_MUL(ml, ml)), GP_MUL(E, E1));
        if (fabs(tmp) <= 3 * GP_DBL_EPSILON * p2) tmp = 0.;
        const double a_mu = 0.5 * tmp / p2;
        const double b_mu = 0.25 / p2;
        double mu = a_mu + b_mu * Q2;
        if (mu < 0)
                mu = 0.;
        else if (mu > 1.)
                mu = 1.;
        return mu;
}

/* polar_ionisation (pumas.c:11965-11976). */
GPD double gp_polar_ionisation(const gp_tables & T, double ki, double kf)
{
        const double nu = ki - kf;
        const double p2 = ki * (ki + 2 * T.mass);
        const double E = ki + T.mass;
        const double c = GP_SUB(p2, GP_MUL(nu, E + GP_ELECTRON_MASS)) /
            sqrt(p2 * GP_SUB(GP_ADD(p2, GP_MUL(nu, nu)),
                          GP_MUL(2 * nu, E)));
        return 0.5 * (1. - c);
}

static __device__ __forceinline__ double gp_polar(const gp_tables & T, gp_event & e, int process,
    const gp_element & el, double ki, double kf)
{
        if (process <= 1)
                return gp_polar_bremsstrahlung(T, e, el, ki, kf);
        else if (process == 2)
                return gp_polar_photonuclear(T, e, el, ki, kf);
        else
                return gp_polar_ionisation(T, ki, kf);
}

/* ------------------------------------------------------------------------ */
/* DEL sampling (pumas.c:5706-6270, 11185-11226).                           */
/* ------------------------------------------------------------------------ */

/* dcs_ionisation_randomise (pumas.c:11185-11226). */
static __device__ __forceinline__ double gp_ionisation_randomise(const gp_tables & T,
    const gp_config & cfg, gp_event & e, const gp_element & el, double K,
    double xlow)
{
        const double P2 = K * (K + 2. * T.mass);
        const double E = K + T.mass;
        const double Wmax = 2. * GP_ELECTRON_MASS * P2 /
            (T.mass * T.mass +
                GP_ELECTRON_MASS * (GP_ELECTRON_MASS + 2. * E));
        if (Wmax < T.cutoff * K) return K;
        double Wmin = (13.6 / 19.2) * el.I;
        const double qlow = K * xlow;
        if (qlow >= Wmin) Wmin = qlow;
        const double E2 = E * E;
        const double beta2 = P2 / E2;
        const double a0 = 0.5 / E2;
        const double a1 = beta2 / Wmax;
        const double p0 = a0 * (Wmax - Wmin);
        const double p2 = 1. / Wmin - 1. / Wmax;
        double q = 0.;
        int trials;
        for (trials = 0; trials < cfg.max_trials; trials++) {
                double z = gp_random(e) * (p0 + p2);
                if (z <= p0) {
                        z /= p0;
                        q = (Wmax - Wmin) * z;
                } else {
                        z = (z - p0) / p2;
                        q = Wmin * Wmax / (Wmax - z * (Wmax - Wmin));
                }
                const double r0 = a0 + 1 / (q * q);
                const double r1 = r0 - a1 / q;
                if (gp_random(e) * r0 <= r1) break;
        }
        if (trials == cfg.max_trials) e.status = GPUMAS_RETURN_INTERNAL_ERROR;
        return K - q;
}

GPD double gp_envelope_norm(double a, double xmin, double xmax)
{
        if (a == 1)
                return gp_log(xmax / xmin);
        else
                return (pow(xmin, 1. - a) - pow(xmax, 1. - a)) / (a - 1.);
}

/* del_randomise_target (pumas.c:6154-6270). Returns the process and sets the
 * target element; in backward mode also the DCS sum as *weight. */
static __device__ __forceinline__ void gp_del_target(const gp_tables & T, const gp_config & cfg,
    gp_event & e, int material, double Q, int & process, int & element,
    double & weight)
{
        int i1;
        double h, dk;
        i1 = gp_index(T, GP_LUT_K, T.K, e.energy);
        if (i1 < 0) {
                i1 = 0;
                h = dk = 0.;
        } else if (i1 >= T.n_energies - 1) {
                i1 = T.n_energies - 1;
                h = dk = 0.;
        } else {
                const double K1 = __ldg(T.K + i1);
                dk = __ldg(T.K + i1 + 1) - K1;
                h = (e.energy - K1) / dk;
        }
        const int ic0 = __ldg(T.comp_start + material);
        const int nc = __ldg(T.elements_in + material);
        if (cfg.direction == GPUMAS_MODE_FORWARD) {
                const double zeta = gp_random(e);
                for (int ic = ic0; ic < ic0 + nc; ic++) {
                        for (int ip = 0; ip < GP_N_DEL; ip++) {
                                const long o =
                                    (long)(ip * T.n_components + ic) *
                                        T.n_energies + i1;
                                const double csf = gp_pchip(h,
                                    __ldg(T.CSf + o), __ldg(T.CSf + o + 1),
                                    __ldg(T.CSf_dK + o) * dk,
                                    __ldg(T.CSf_dK + o + 1) * dk);
                                if (!(zeta > csf)) {
                                        element = __ldg(T.comp_element + ic);
                                        process = ip;
                                        return;
                                }
                        }
                }
                /* Not reached for consistent tables (pumas.c:6209). */
                element = __ldg(T.comp_element + ic0 + nc - 1);
                process = GP_N_DEL - 1;
                e.status = GPUMAS_RETURN_INTERNAL_ERROR;
                return;
        }
        double stot = 0.;
        for (int ip = 0; ip < GP_N_DEL; ip++) {
                for (int ic = ic0; ic < ic0 + nc; ic++) {
                        const gp_element & el =
                            T.element[__ldg(T.comp_element + ic)];
                        const double d = gp_dcs_evaluate(T, ip, el, e.energy, Q);
                        stot += d * __ldg(T.comp_fraction + ic);
                }
        }
        if (stot == 0.) {
                weight = 0.;
                return;
        }
        weight = stot;
        if (cfg.scattering == GPUMAS_MODE_DISABLED) {
                element = T.n_elements;
                process = GP_N_DEL;
                return;
        }
        double zeta = 0.;
        int trials;
        for (trials = 0; trials < cfg.max_trials; trials++) {
                zeta = gp_random(e) * stot;
                if ((zeta > 0.) && (zeta < stot)) break;
        }
        if (trials == cfg.max_trials) e.status = GPUMAS_RETURN_INTERNAL_ERROR;
        /* The energy transfer and the weight share a union in the reference
         * (struct del_info, pumas.c:643-655): the selection below evaluates
         * the DCS at an energy transfer equal to stot (pumas.c:6250). */
        const double Q_union = stot;
        double s = 0.;
        for (int ic = ic0; ic < ic0 + nc; ic++) {
                const int iel = __ldg(T.comp_element + ic);
                const gp_element & el = T.element[iel];
                for (int ip = 0; ip < GP_N_DEL; ip++) {
                        const double si =
                            gp_dcs_evaluate(T, ip, el, e.energy, Q_union) *
                            __ldg(T.comp_fraction + ic);
                        s += si;
                        if (!(zeta > s)) {
                                element = iel;
                                process = ip;
                                return;
                        }
                }
        }
        element = __ldg(T.comp_element + ic0 + nc - 1);
        process = GP_N_DEL - 1;
        e.status = GPUMAS_RETURN_INTERNAL_ERROR;
}

/* del_randomise_forward (pumas.c:5912-6017). Returns true if a polar angle
 * is to be sampled. */
static __device__ __forceinline__ bool gp_del_forward(const gp_tables & T, const gp_config & cfg,
    gp_event & e, int material, int & process, int & target)
{
        if (e.energy <= __ldg(T.Kt + material)) return false;
        int ip = 0, iel = 0;
        double w = 0.;
        gp_del_target(T, cfg, e, material, 0., ip, iel, w);
        const gp_element & el = T.element[iel];
        target = iel;
        process = ip;
        if (ip == 3) {
                e.energy = gp_ionisation_randomise(
                    T, cfg, e, el, e.energy, T.cutoff);
                return true;
        }
        double qmin, qmax;
        if (ip == 2) {
                gp_photonuclear_range(T.mass, e.energy, qmin, qmax);
        } else {
                qmax = e.energy + T.mass * el.qmax_m_pair;
                qmin = (ip == 0) ? 0. : 4. * GP_ELECTRON_MASS;
        }
        double xmin = qmin / e.energy;
        if (xmin < T.cutoff) xmin = T.cutoff;
        const double xmax = qmax / e.energy;
        if (xmin >= xmax) return false;

        double a0, a1, b0, b1, p0;
        const int imax = T.n_energies - 1;
        const float * env = T.DCS_env +
            2 * ((long)(ip * T.n_elements + el.index) * T.n_energies);
        if (e.energy >= __ldg(T.K + imax)) {
                a0 = (double)__ldg(env + 2 * imax);
                b0 = (double)__ldg(env + 2 * imax + 1);
                p0 = 1.;
                a1 = b1 = 0.;
        } else {
                const int row = gp_index(T, GP_LUT_K, T.K, e.energy);
                a0 = (double)__ldg(env + 2 * row);
                b0 = (double)__ldg(env + 2 * row + 1);
                a1 = (double)__ldg(env + 2 * row + 2);
                b1 = (double)__ldg(env + 2 * row + 3);
                const double k0 = __ldg(T.K + row);
                const double k1 = __ldg(T.K + row + 1);
                const double h1 = (e.energy - k0) / (k1 - k0);
                const double h0 = 1. - h1;
                b0 *= h0;
                b1 *= h1;
                p0 = gp_envelope_norm(a0, xmin, xmax) * b0;
                const double p1 = gp_envelope_norm(a1, xmin, xmax) * b1;
                p0 /= p0 + p1;
        }
        double x = 0.;
        int i;
        for (i = 0; i < 100; i++) {
                double u = gp_random(e);
                double a;
                if (u < p0) {
                        a = a0;
                        u = u / p0;
                } else {
                        a = a1;
                        u = (u - p0) / (1. - p0);
                }
                if (a == 1) {
                        x = xmin * gp_exp(u * gp_log(xmax / xmin));
                } else {
                        const double am = a - 1.;
                        const double pmin = pow(xmin, -am);
                        const double pmax = pow(xmax, -am);
                        x = pow(pmin - u * (pmin - pmax), -1. / am);
                }
                const double penv = b0 * pow(x, -a0) + b1 * pow(x, -a1);
                const double d = gp_dcs_evaluate(T, ip, el, e.energy,
                    e.energy * x);
                if (gp_random(e) * penv <= d) break;
        }
        if (i == 100) return false;
        e.energy *= (1. - x);
        return true;
}

/* del_randomise_reverse (pumas.c:6036-6093) with the power law sampling
 * of del_randomise_power_law (pumas.c:6109-6138), alpha = 2. */
static __device__ __forceinline__ bool gp_del_reverse(const gp_tables & T, const gp_config & cfg,
    gp_event & e, int material, int & process, int & target)
{
        const double lnq0 = -gp_log(T.cutoff);
        const double kt = __ldg(T.Kt + material);
        const double kf = e.energy;
        const double pCEL =
            (kf >= kt) ? 0. : lnq0 / (lnq0 + gp_log(kt / (kt - kf)));
        if (pCEL && (gp_random(e) < pCEL)) {
                e.weight /= pCEL;
                return false;
        }
        const double xf =
            (kf >= kt * (1. - T.cutoff)) ? T.cutoff : 1. - kf / kt;
        double xmax;
        const double m1 = T.mass - GP_ELECTRON_MASS;
        if (e.energy < 0.5 * m1 * m1 / GP_ELECTRON_MASS) {
                const double m2 = T.mass + GP_ELECTRON_MASS;
                xmax = 2. * GP_ELECTRON_MASS * (e.energy + 2. * T.mass) /
                    (m2 * m2);
                if (xmax < xf)
                        return false;
                else if (xmax > 1.)
                        xmax = 1.;
        } else {
                xmax = 1.;
        }
        double r = 0., w_bias = 0.;
        {
                const double alpha = 2.0;
                const double a1 = 1. - alpha;
                const double x0 = pow(xf, a1);
                const double x1 = pow(xmax, a1);
                int trials;
                for (trials = 0; trials < cfg.max_trials; trials++) {
                        const double z = gp_random(e);
                        const double tmp = x0 + z * (x1 - x0);
                        r = pow(tmp, 1. / a1);
                        if ((r < xf) || (r >= xmax)) continue;
                        w_bias = (x1 - x0) * r / (a1 * tmp);
                        break;
                }
                if (trials == cfg.max_trials) {
                        e.status = GPUMAS_RETURN_INTERNAL_ERROR;
                        return false;
                }
                r = 1. - r;
        }
        w_bias /= r;
        e.energy /= r;
        int ip = 0, iel = 0;
        double weight = 0.;
        gp_del_target(T, cfg, e, material, e.energy - kf, ip, iel, weight);
        if (weight <= 0) {
                e.weight = 0.;
                return false;
        }
        e.weight *= w_bias * weight /
            (gp_del_cross_section(T, material, kf) * (1. - pCEL));
        process = ip;
        if (cfg.scattering == GPUMAS_MODE_DISABLED) return false;
        target = iel;
        return true;
}

/* transport_do_del (pumas.c:5706-5757). */
/* A sampled DEL whose polar angle is still to be drawn. */
struct gp_polar_job {
        int process;   /* -1 if no polar angle is to be sampled */
        int target;
        double ki, kf; /* initial and final energies, ki >= kf */
};

/* First part of transport_do_del (pumas.c:5706-5745): the energy loss and
 * the event flag. Returns in *job the pending polar angle, if any. */
static __device__ __forceinline__ void gp_do_del_energy(const gp_tables & T,
    const gp_config & cfg, gp_event & e, int material, gp_polar_job & job)
{
        double ki, kf;
        int process = -1, target = 0;
        bool polar;
        if (cfg.direction == GPUMAS_MODE_FORWARD) {
                ki = e.energy;
                polar = gp_del_forward(T, cfg, e, material, process, target);
                kf = e.energy;
        } else {
                kf = e.energy;
                polar = gp_del_reverse(T, cfg, e, material, process, target);
                ki = e.energy;
        }
        if (process < 0) {
                e.step_event = (e.weight > 0) ? GPUMAS_EVENT_NONE :
                                                GPUMAS_EVENT_WEIGHT;
        } else {
                e.step_event = (process == 0) ?
                    GPUMAS_EVENT_VERTEX_BREMSSTRAHLUNG :
                    (process == 1) ? GPUMAS_EVENT_VERTEX_PAIR_CREATION :
                    (process == 2) ? GPUMAS_EVENT_VERTEX_PHOTONUCLEAR :
                    (process == 3) ? GPUMAS_EVENT_VERTEX_DELTA_RAY :
                                     GPUMAS_EVENT_VERTEX;
        }
        job.process = -1;
        if ((cfg.scattering == GPUMAS_MODE_MIXED) && polar) {
                if (kf > ki) {
                        const double tmp = kf;
                        kf = ki;
                        ki = tmp;
                }
                job.process = process;
                job.target = target;
                job.ki = ki;
                job.kf = kf;
        }
}

/* Second part of transport_do_del (pumas.c:5746-5756): the polar angle and
 * the rotation of the direction. */
static __device__ __forceinline__ void gp_do_del_polar(const gp_tables & T,
    gp_event & e, const gp_polar_job & job)
{
        if (job.process < 0) return;
        const double mu = gp_polar(T, e, job.process, T.element[job.target],
            job.ki, job.kf);
        gp_rotate(e, mu);
}

/* transport_do_del (pumas.c:5706-5757). */
static __device__ __forceinline__ void gp_do_del(const gp_tables & T,
    const gp_config & cfg, gp_event & e, int material)
{
        gp_polar_job job;
        gp_do_del_energy(T, cfg, e, material, job);
        gp_do_del_polar(T, e, job);
}

/* ------------------------------------------------------------------------ */
/* Elastic hard scattering (transport_do_ehs, pumas.c:5768-5885).           */
/* ------------------------------------------------------------------------ */
static __device__ __forceinline__ void gp_do_ehs(const gp_tables & T, const gp_config & cfg,
    gp_event & e, int material)
{
        const double kinetic = e.energy;
        double mu0 = 0., invlb1 = 0.;
        gp_table_get_msc(T, cfg.energy_loss, material, kinetic, mu0, invlb1);
        const int n_el = __ldg(T.elements_in + material);
        const int ic0 = __ldg(T.comp_start + material);
        const double fspin = gp_coulomb_spin_factor(T.mass, kinetic);

        /* Choice of the hard scatterer: the restricted cross sections are
         * only needed for compound materials. */
        int ihard = n_el - 1;
        if (n_el > 1) {
                double cs_hard[GP_MAX_COMPONENTS];
                double cs_tot = 0.;
                for (int i = 0; i < n_el; i++) {
                        const gp_element & el =
                            T.element[__ldg(T.comp_element + ic0 + i)];
                        double kinetic0, fCM[2], amplitude[3], screening[3];
                        double N, a[3], b[3], c[4];
                        gp_coulomb_frame_parameters(
                            el.Ma, T.mass, kinetic, kinetic0, fCM);
                        const int np = gp_coulomb_screening(el, T.mass,
                            kinetic, kinetic0, amplitude, screening, N);
                        gp_coulomb_pole_reduction(
                            np, amplitude, screening, N, a, b, c);
                        const double normalisation =
                            __ldg(T.comp_fraction + ic0 + i) /
                            gp_coulomb_normalisation(
                                el.Z, el.A, T.mass, kinetic, kinetic0);
                        cs_hard[i] = normalisation *
                            gp_coulomb_restricted_cs(
                                mu0, fspin, np, screening, N, a, b, c);
                        cs_tot += cs_hard[i];
                }
                const double cc0 = gp_random(e) * cs_tot;
                double cs = 0.;
                for (int i = 0; i < n_el; i++) {
                        cs += cs_hard[i];
                        if (cs >= cc0) {
                                ihard = i;
                                break;
                        }
                }
        } else {
                /* One element: the draw is consumed, the choice forced. */
                gp_random(e);
        }

        const gp_element & el = T.element[__ldg(T.comp_element + ic0 + ihard)];
        double kinetic0, fCM[2], amplitude[3], screening[3], N;
        gp_coulomb_frame_parameters(el.Ma, T.mass, kinetic, kinetic0, fCM);
        const int np = gp_coulomb_screening(
            el, T.mass, kinetic, kinetic0, amplitude, screening, N);
        const int n = np - 1;
        double A = screening[0];
        for (int i = 1; i < 3; i++) {
                if (i >= n) break;
                if (screening[i] < A) A = screening[i];
        }
        double mu1 = mu0;
        int trials;
        for (trials = 0; trials < cfg.max_trials; trials++) {
                const double zeta = gp_random(e);
                const double tmp = 1. + A - zeta * (1 - mu0);
                if (tmp <= 0.) continue;
                mu1 = (A + mu0) * (A + 1.) / tmp - A;
                if (mu1 < mu0)
                        mu1 = mu0;
                else if (mu1 > 1.)
                        mu1 = 1;
                double ratio = 0.;
                for (int k = 0; k < 3; k++) {
                        if (k >= n) break;
                        ratio += amplitude[k] * (A + mu1) / (screening[k] + mu1);
                }
                ratio *= gp_coulomb_nuclear_form_factor(mu1, N);
                ratio *= ratio * (1. - fspin * mu1);
                if (gp_random(e) <= ratio) break;
        }
        if (trials == cfg.max_trials) e.status = GPUMAS_RETURN_INTERNAL_ERROR;
        const double gamma = fCM[0];
        const double tau = fCM[1];
        double mu;
        if (mu1 > 1E-06) {
                const double a = gamma * (tau + 1. - 2. * mu1);
                const double ct_h = a / sqrt(4. * mu1 * (1. - mu1) + a * a);
                mu = 0.5 * (1. - ct_h);
        } else {
                const double d = gamma * (1. + tau);
                mu = mu1 / (d * d);
        }
        gp_rotate(e, mu);
}

/* ------------------------------------------------------------------------ */
/* Stepping (pumas.c:5194-5696, 6296-7005).                                 */
/* ------------------------------------------------------------------------ */

/* step_fluctuate (pumas.c:6943-7005). */
static __device__ __forceinline__ void gp_fluctuate(const gp_tables & T, const gp_config & cfg,
    gp_event & e, int material, double Xtot, double dX, double & kf,
    double & ratio)
{
        const int scheme = cfg.energy_loss;
        const double sgn = (cfg.direction == GPUMAS_MODE_FORWARD) ? 1. : -1.;
        double k1, r = 0.;
        k1 = gp_cel_kinetic_energy(T, scheme, material, Xtot - sgn * dX);
        const double dk0 = fabs(e.energy - k1);
        if ((k1 > 0.) && (dk0 > 0.)) {
                const double Omega0 = gp_cel_straggling(T, material, e.energy);
                const double Omega1 = gp_cel_straggling(T, material, k1);
                double dk12 = 0.5 * dX * (Omega0 + Omega1);
                if (dX > 5E-02 * Xtot) {
                        const double de1 =
                            gp_cel_energy_loss(T, scheme, material, k1);
                        const double de0 =
                            gp_cel_energy_loss(T, scheme, material, e.energy);
                        dk12 *= 1. + sgn * dX / dk0 * (de1 - de0);
                }
                const double dk1 = sqrt(dk12);
                if (dk0 >= 3. * dk1) {
                        double u;
                        int trials = 0;
                        do {
                                u = gp_randn(e);
                        } while ((fabs(u) > 3.) &&
                            (++trials < cfg.max_trials));
                        if (trials == cfg.max_trials)
                                e.status = GPUMAS_RETURN_INTERNAL_ERROR;
                        u *= 1. / 1.015387;
                        k1 += u * dk1;
                } else if (dk0 >= 1.7320508 * dk1) {
                        const double u = 1.7320508 * (1. - 2. * gp_random(e));
                        k1 += u * dk1;
                } else {
                        const double dk32 = 3. * dk12;
                        const double dk02 = dk0 * dk0;
                        const double a =
                            1. - (dk32 - dk02) / (dk32 + 3. * dk02);
                        if (gp_random(e) <= a) {
                                const double b =
                                    0.5 * (dk32 + 3. * dk02) / dk0;
                                const double u = gp_random(e);
                                k1 = e.energy - sgn * b * u;
                                if (k1 < 0.) k1 = 0.;
                        } else {
                                k1 = e.energy;
                        }
                }
                r = fabs(e.energy - k1) / dk0;
        }
        if (r == 0.) r = 1.;
        kf = k1;
        ratio = r;
}

/* transport_limit (pumas.c:5569-5696). */
static __device__ __forceinline__ void gp_limit(const gp_tables & T, const gp_config & cfg,
    gp_event & e, int material, double Xi, double Xf, double & grammage_max)
{
        e.step_event = e.step_foreseen = GPUMAS_EVENT_NONE;
        if (e.weight <= 0.) {
                e.step_event = GPUMAS_EVENT_WEIGHT;
                return;
        }
        if (cfg.direction == GPUMAS_MODE_FORWARD) {
                const double kinetic_min =
                    (cfg.event & GPUMAS_EVENT_LIMIT_ENERGY) ?
                    cfg.limit_energy : 0.;
                if (e.energy <= kinetic_min) {
                        e.step_event = GPUMAS_EVENT_LIMIT_ENERGY;
                        return;
                }
        } else if ((cfg.event & GPUMAS_EVENT_LIMIT_ENERGY) &&
            (e.energy >= cfg.limit_energy)) {
                e.step_event = GPUMAS_EVENT_LIMIT_ENERGY;
                return;
        }
        if (cfg.event & GPUMAS_EVENT_LIMIT_GRAMMAGE) {
                grammage_max = cfg.limit_grammage;
                e.step_foreseen = GPUMAS_EVENT_LIMIT_GRAMMAGE;
        } else {
                grammage_max = 0.;
        }
        const int scheme = cfg.energy_loss;
        if (scheme == GPUMAS_MODE_DISABLED) {
                if (cfg.scattering == GPUMAS_MODE_MIXED) {
                        const double X = Xi -
                            gp_coulomb_ehs_length(T, material, e.energy) *
                                gp_log(gp_random(e));
                        if ((grammage_max == 0.) || (X < grammage_max)) {
                                grammage_max = X;
                                e.step_foreseen = GPUMAS_EVENT_VERTEX_COULOMB;
                                return;
                        }
                }
                return;
        }
        const double sgn = (cfg.direction == GPUMAS_MODE_FORWARD) ? 1. : -1.;
        int foreseen = GPUMAS_EVENT_NONE;
        double kinetic_limit = 0.;
        if (scheme == GPUMAS_MODE_MIXED) {
                for (int i = 0; i < 1000; i++) {
                        const double zeta = gp_random(e);
                        if ((zeta <= 0.) || (zeta >= 1.)) continue;
                        const double nI =
                            gp_del_interaction_length(T, material, e.energy) +
                            sgn * gp_log(zeta);
                        if (nI <= 0.) break;
                        const double k = gp_del_kinetic_from_interaction_length(
                            T, material, nI);
                        if (cfg.direction == GPUMAS_MODE_FORWARD) {
                                if (k >= e.energy) continue;
                        } else {
                                if (k <= e.energy) continue;
                        }
                        if ((cfg.direction == GPUMAS_MODE_BACKWARD) ||
                            (k > __ldg(T.Kt + material))) {
                                kinetic_limit = k;
                                foreseen = GPUMAS_EVENT_VERTEX_DEL;
                        }
                        break;
                }
        }
        if ((scheme < GPUMAS_MODE_STRAGGLED) &&
            (cfg.scattering == GPUMAS_MODE_MIXED)) {
                const double nI = gp_ehs_interaction_length(
                                      T, scheme, material, e.energy) +
                    sgn * gp_log(gp_random(e));
                if (nI > 0.) {
                        const double k = gp_ehs_kinetic_from_interaction_length(
                            T, scheme, material, nI);
                        if ((kinetic_limit <= 0.) ||
                            ((cfg.direction == GPUMAS_MODE_FORWARD) &&
                                (k > kinetic_limit)) ||
                            ((cfg.direction == GPUMAS_MODE_BACKWARD) &&
                                (k < kinetic_limit))) {
                                kinetic_limit = k;
                                foreseen = GPUMAS_EVENT_VERTEX_COULOMB;
                        }
                }
        }
        if (foreseen == GPUMAS_EVENT_NONE) return;
        const double X = Xi + sgn * (Xf - gp_cel_grammage(
                                            T, scheme, material, kinetic_limit));
        if ((grammage_max <= 0) || (X < grammage_max)) {
                grammage_max = X;
                e.step_foreseen = foreseen;
        }
}

/* Magnetic deflection at the end of a step (pumas.c:6833-6911): the
 * direction turns by the mean of the Larmor angles of the step's two end
 * points, about the mean of their deflection directions. */
GPD void gp_step_deflect(const gp_tables & T, const gp_config & cfg,
    gp_event & e, const gp_loc & loc, const double * Bi, double h_int,
    double momentum, double step, double rLarmor0, const double * uT0)
{
        double rLarmor1 = 0., uT1[3] = { 0., 0., 0. };
        if (loc.magnetized) {
                double B[3] = { loc.magnet[0], loc.magnet[1], loc.magnet[2] };
                int magnetized = loc.magnetized;
                if (h_int > 0.) {
                        B[0] = GP_ADD(Bi[0], GP_MUL(h_int, GP_SUB(B[0], Bi[0])));
                        B[1] = GP_ADD(Bi[1], GP_MUL(h_int, GP_SUB(B[1], Bi[1])));
                        B[2] = GP_ADD(Bi[2], GP_MUL(h_int, GP_SUB(B[2], Bi[2])));
                        /* The reference's test, kept as it is: a truncated
                         * step (h_int > 0) takes no end point deflection
                         * (pumas.c:6843-6844). */
                        magnetized = (GP_ADD(GP_ADD(GP_MUL(B[0], B[0]),
                            GP_MUL(B[1], B[1])), GP_MUL(B[2], B[2])) == 0.);
                }
                if (magnetized != 0) {
                        const double p = (e.energy <= 0) ? momentum :
                            sqrt(e.energy * (e.energy + 2. * T.mass));
                        rLarmor1 = gp_larmor(e.dir, B, p, uT1);
                }
        }
        if ((rLarmor0 <= 0.) && (rLarmor1 <= 0.)) return;
        const double u[3] = { e.dir[0], e.dir[1], e.dir[2] };
        const double cs = GP_MUL(e.charge, step);
        const double theta0 = (rLarmor0 > 0.) ? cs / rLarmor0 : 0.;
        const double theta1 = (rLarmor1 > 0.) ? cs / rLarmor1 : 0.;
        double theta = GP_MUL(0.5, GP_ADD(theta0, theta1));
        if (cfg.direction == GPUMAS_MODE_BACKWARD) theta = -theta;
        double c = cos(theta);
        double sn = sin(theta);
        double v[3];
        for (int i = 0; i < 3; i++) v[i] = GP_MUL(0.5, GP_ADD(uT0[i], uT1[i]));
        double nrmv = GP_ADD(GP_ADD(GP_MUL(v[0], v[0]), GP_MUL(v[1], v[1])),
            GP_MUL(v[2], v[2]));
        if (nrmv > 0.) {
                nrmv = 1. / sqrt(nrmv);
                for (int i = 0; i < 3; i++) v[i] = GP_MUL(v[i], nrmv);
        } else {
                c = 1.;
                sn = 0.;
        }
        for (int i = 0; i < 3; i++)
                e.dir[i] = GP_ADD(GP_MUL(c, u[i]), GP_MUL(sn, v[i]));
        const double norm = 1. / sqrt(GP_ADD(GP_ADD(GP_MUL(e.dir[0], e.dir[0]),
            GP_MUL(e.dir[1], e.dir[1])), GP_MUL(e.dir[2], e.dir[2])));
        for (int i = 0; i < 3; i++) e.dir[i] = GP_MUL(e.dir[i], norm);
}

/* step_transport (pumas.c:6296-6925). Sets e.step_event and returns the
 * end step medium. With locals (loc not NULL) the density at the end of the
 * step goes to loc->density, and a magnetic field bends the step. */
static __device__ __forceinline__ int gp_step(const gp_tables & T, const gp_config & cfg,
    const gpumas_geometry & g, gp_event & e, int straight, int medium,
    int material, double density, double grammage_max,
    double step_max_medium, gp_loc * loc = NULL)
{
        const int scheme = cfg.energy_loss;
        const double density_i = 1. / density;
        const double momentum = sqrt(e.energy * (e.energy + 2. * T.mass));
        const int tmp_scheme =
            (scheme == GPUMAS_MODE_DISABLED) ? GPUMAS_MODE_CSDA : scheme;
        const double Xtot = gp_cel_grammage(T, tmp_scheme, material, e.energy);

        double step_loc;
        double invlb1 = 0.;
        double rLarmor0 = 0., uT0[3] = { 0., 0., 0. };
        if (!straight) {
                double r = cfg.accuracy;
                const double k_threshold = 1E+09;
                if ((scheme == GPUMAS_MODE_STRAGGLED) &&
                    (e.energy > k_threshold)) {
                        double f = k_threshold / e.energy;
                        if (f < 0.1) f = 0.1;
                        r *= f;
                }
                step_loc = r * density_i * Xtot;
                if (cfg.scattering == GPUMAS_MODE_MIXED) {
                        if (e.step_first != 0) {
                                double mu0;
                                gp_table_get_msc(T, scheme, material,
                                    e.energy, mu0, invlb1);
                                invlb1 *= density;
                        } else
                                invlb1 = e.step_invlb1;
                        const double stepT = cfg.accuracy / invlb1;
                        if (stepT < step_loc) step_loc = stepT;
                }
                if ((loc != NULL) && loc->magnetized) {
                        rLarmor0 = gp_larmor(e.dir, loc->magnet, momentum, uT0);
                        if (rLarmor0 > 0.) {
                                const double stepM = cfg.accuracy * rLarmor0;
                                if (stepM < step_loc) step_loc = stepM;
                        }
                }
        } else {
                if (grammage_max <= 0.)
                        step_loc = 1E+09 * density_i;
                else
                        step_loc = grammage_max * density_i;
        }
        e.step_first = 0;
        if (step_loc < GP_STEP_MIN) step_loc = GP_STEP_MIN;
        double step = (step_max_medium <= 0) ?
            step_loc :
            (step_max_medium < step_loc ? step_max_medium : step_loc);
        if ((loc != NULL) && (loc->step_max > 0.) && (step > loc->step_max))
                step = loc->step_max;

        int out_medium = medium;
        int event = GPUMAS_EVENT_NONE;
        if (cfg.event & GPUMAS_EVENT_LIMIT_DISTANCE) {
                const double d = cfg.limit_distance - e.distance;
                if (d <= step) {
                        step = d;
                        event = GPUMAS_EVENT_LIMIT_DISTANCE;
                }
        }
        const double sgn = (cfg.direction == GPUMAS_MODE_FORWARD) ? 1. : -1.;
        const double sd0 = sgn * e.dir[0], sd1 = sgn * e.dir[1],
                     sd2 = sgn * e.dir[2];
        /* Separate roundings, as the reference's position update
         * (pumas.c:6416-6418): the position accumulates over the track. */
        e.pos[0] = GP_ADD(e.pos[0], GP_MUL(step, sd0));
        e.pos[1] = GP_ADD(e.pos[1], GP_MUL(step, sd1));
        e.pos[2] = GP_ADD(e.pos[2], GP_MUL(step, sd2));

        int end_medium = gp_locate(g, e);
        /* Where the end step locals are evaluated when the step crosses a
         * boundary: the last point inside the medium (pumas.c:6440-6492). */
        double pl[3];
        if (end_medium != medium) {
                /* Boundary check of a PUMAS_STEP_CHECK geometry
                 * (pumas.c:6425-6485). */
                const double step_min = (step < GP_STEP_MIN) ? step : GP_STEP_MIN;
                const double pi0 = e.pos[0], pi1 = e.pos[1], pi2 = e.pos[2];
                double s1 = 0., s2 = -step_min;
                e.pos[0] = GP_ADD(pi0, GP_MUL(s2, sd0));
                e.pos[1] = GP_ADD(pi1, GP_MUL(s2, sd1));
                e.pos[2] = GP_ADD(pi2, GP_MUL(s2, sd2));
                int tmp_medium = gp_locate(g, e);
                if (tmp_medium != medium) {
                        if (tmp_medium != end_medium) end_medium = tmp_medium;
                        s1 = s2;
                        s2 = -step;
                        while (fabs(s1 - s2) > GP_STEP_MIN) {
                                double s3 = 0.5 * (s1 + s2);
                                e.pos[0] = GP_ADD(pi0, GP_MUL(s3, sd0));
                                e.pos[1] = GP_ADD(pi1, GP_MUL(s3, sd1));
                                e.pos[2] = GP_ADD(pi2, GP_MUL(s3, sd2));
                                tmp_medium = gp_locate(g, e);
                                if (tmp_medium == medium) {
                                        s2 = s3;
                                } else {
                                        s1 = s3;
                                        if (tmp_medium != end_medium)
                                                end_medium = tmp_medium;
                                }
                        }
                        step += s1;
                        if (loc != NULL) {
                                pl[0] = GP_ADD(pi0, GP_MUL(s2, sd0));
                                pl[1] = GP_ADD(pi1, GP_MUL(s2, sd1));
                                pl[2] = GP_ADD(pi2, GP_MUL(s2, sd2));
                        }
                        e.pos[0] = GP_ADD(pi0, GP_MUL(s1, sd0));
                        e.pos[1] = GP_ADD(pi1, GP_MUL(s1, sd1));
                        e.pos[2] = GP_ADD(pi2, GP_MUL(s1, sd2));
                } else {
                        if (loc != NULL) {
                                pl[0] = e.pos[0];
                                pl[1] = e.pos[1];
                                pl[2] = e.pos[2];
                        }
                        e.pos[0] = pi0;
                        e.pos[1] = pi1;
                        e.pos[2] = pi2;
                }
                event = GPUMAS_EVENT_MEDIUM;
                out_medium = end_medium;
        }

        /* End step locals (pumas.c:6488-6503). */
        double density1 = density;
        double Bi[3] = { 0., 0., 0. };
        if (loc != NULL) {
                if (loc->magnetized) {
                        Bi[0] = loc->magnet[0];
                        Bi[1] = loc->magnet[1];
                        Bi[2] = loc->magnet[2];
                }
                if (loc->step_max > 0.) {
                        double pe[3] = { e.pos[0], e.pos[1], e.pos[2] };
                        if (event & GPUMAS_EVENT_MEDIUM) {
                                e.pos[0] = pl[0];
                                e.pos[1] = pl[1];
                                e.pos[2] = pl[2];
                        }
                        loc->step_max = gp_set_locals(
                            T, cfg, e, medium, density1, *loc);
                        e.pos[0] = pe[0];
                        e.pos[1] = pe[1];
                        e.pos[2] = pe[2];
                        if (density1 <= 0.) {
                                e.status = GPUMAS_RETURN_DENSITY_ERROR;
                                return out_medium;
                        }
                }
                loc->density = density1;
        }
        double k1 = e.energy, dk = 0.;
        const double dX = 0.5 * step * (density + density1);
        if ((scheme >= GPUMAS_MODE_CSDA) && (scheme <= GPUMAS_MODE_MIXED)) {
                const double X = Xtot - sgn * dX;
                if ((cfg.direction == GPUMAS_MODE_FORWARD) &&
                    (X <= e.step_X_limit)) {
                        k1 = (cfg.event & GPUMAS_EVENT_LIMIT_ENERGY) ?
                            cfg.limit_energy : 0.;
                        const double grammage =
                            e.grammage + Xtot - e.step_X_limit;
                        if ((grammage_max <= 0.) || (grammage < grammage_max)) {
                                grammage_max = grammage;
                                event = GPUMAS_EVENT_LIMIT_ENERGY;
                        }
                } else if ((cfg.direction == GPUMAS_MODE_BACKWARD) &&
                    (e.step_X_limit > 0.) && (X > e.step_X_limit)) {
                        k1 = (cfg.event & GPUMAS_EVENT_LIMIT_ENERGY) ?
                            cfg.limit_energy : 0.;
                        const double grammage =
                            e.grammage + e.step_X_limit - Xtot;
                        if ((grammage_max <= 0.) || (grammage < grammage_max)) {
                                grammage_max = grammage;
                                event = GPUMAS_EVENT_LIMIT_ENERGY;
                        }
                } else if (dX < GP_EPSILON_X * Xtot) {
                        k1 -= sgn * gp_cel_energy_loss(T, scheme, material, k1) *
                            dX;
                        if ((cfg.event & GPUMAS_EVENT_LIMIT_ENERGY) &&
                            (cfg.limit_energy > 0.)) {
                                if (((cfg.direction == GPUMAS_MODE_FORWARD) &&
                                        (k1 < cfg.limit_energy)) ||
                                    ((cfg.direction == GPUMAS_MODE_BACKWARD) &&
                                        (k1 > cfg.limit_energy))) {
                                        k1 = cfg.limit_energy;
                                        event = GPUMAS_EVENT_LIMIT_ENERGY;
                                }
                        } else if (k1 < 0.) {
                                k1 = 0.;
                        }
                } else {
                        k1 = gp_cel_kinetic_energy(T, scheme, material, X);
                }
        } else if (scheme == GPUMAS_MODE_STRAGGLED) {
                double ratio;
                gp_fluctuate(T, cfg, e, material, Xtot, dX, k1, ratio);
                dk = fabs(e.energy - k1);
                double kinetic_limit = -1.;
                if (cfg.direction == GPUMAS_MODE_FORWARD) {
                        const double kinetic_min =
                            (cfg.event & GPUMAS_EVENT_LIMIT_ENERGY) ?
                            cfg.limit_energy : 0.;
                        if (k1 <= kinetic_min) kinetic_limit = kinetic_min;
                } else {
                        if ((cfg.event & GPUMAS_EVENT_LIMIT_ENERGY) &&
                            (k1 >= cfg.limit_energy))
                                kinetic_limit = cfg.limit_energy;
                }
                if (kinetic_limit >= 0.) {
                        const double grammage = e.grammage +
                            fabs(e.energy - kinetic_limit) / dk * dX;
                        k1 = kinetic_limit;
                        if ((grammage_max <= 0.) || (grammage < grammage_max)) {
                                grammage_max = grammage;
                                event = GPUMAS_EVENT_LIMIT_ENERGY;
                        }
                }
                double Xmax = dX;
                if (grammage_max > 0.) {
                        const double dX1 = grammage_max - e.grammage;
                        if (Xmax > dX1) Xmax = dX1;
                }
                double k_x = -1.;
                do {
                        /* DEL candidate, thinned (pumas.c:6600-6621). */
                        double xs_del =
                            gp_del_cross_section(T, material, e.energy);
                        const double tmp_del =
                            gp_del_cross_section(T, material, k1);
                        if (tmp_del > xs_del) xs_del = tmp_del;
                        if (xs_del <= 0.) break;
                        /* Candidates beyond the step, most of them, are
                         * ruled out in single precision (gp_math.cuh) with
                         * the same decision as below. */
                        const double u_del = gp_random(e);
                        if (gp_neglog_beyond(u_del, 1., Xmax, xs_del)) break;
                        const double X_del = -gp_log(u_del) / xs_del;
                        if (X_del >= Xmax) break;
                        const double k_h = gp_cel_kinetic_energy(
                            T, scheme, material, Xtot - sgn * X_del);
                        const double k_del =
                            e.energy - sgn * ratio * fabs(e.energy - k_h);
                        if (k_del <= 0.) break;
                        const double r =
                            gp_del_cross_section(T, material, k_del) / xs_del;
                        if (gp_random(e) > r) break;
                        k_x = k_del;
                        Xmax = X_del;
                        event = GPUMAS_EVENT_VERTEX_DEL;
                } while (0);
                if (cfg.scattering == GPUMAS_MODE_MIXED) do {
                        /* EHS candidate, thinned (pumas.c:6623-6656). */
                        double kmin, kmax;
                        if (k1 <= e.energy)
                                kmin = k1, kmax = e.energy;
                        else
                                kmax = k1, kmin = e.energy;
                        if (kmin < __ldg(T.K + 1)) {
                                const double tmp = kmin;
                                kmin = kmax, kmax = tmp;
                        }
                        const double lb_ehs =
                            gp_coulomb_ehs_length(T, material, kmin);
                        if (lb_ehs <= 0.) break;
                        const double u_ehs = gp_random(e);
                        if (gp_neglog_beyond(u_ehs, lb_ehs, Xmax, 1.)) break;
                        const double X_ehs = -gp_log(u_ehs) * lb_ehs;
                        if (X_ehs >= Xmax) break;
                        const double k_h = gp_cel_kinetic_energy(
                            T, scheme, material, Xtot - sgn * X_ehs);
                        const double k_ehs =
                            e.energy - sgn * ratio * fabs(e.energy - k_h);
                        if (k_ehs <= 0.) break;
                        const double r =
                            gp_coulomb_ehs_length(T, material, k_ehs) / lb_ehs;
                        if ((r <= 0.) || (gp_random(e) > 1. / r)) break;
                        k_x = k_ehs;
                        Xmax = X_ehs;
                        event = GPUMAS_EVENT_VERTEX_COULOMB;
                } while (0);
                if (k_x >= 0.) {
                        k1 = k_x;
                        grammage_max = e.grammage + Xmax;
                }
        }

        const double Xi = e.grammage;
        e.grammage += dX;
        const double sf0 = step;
        double h_int = 0.;
        if ((grammage_max > 0.) && (e.grammage >= grammage_max)) {
                const double dX_ = grammage_max - Xi;
                if (loc == NULL) {
                        step = dX_ * density_i;
                } else if ((fabs(density - density1) <= GP_FLT_EPSILON) ||
                    (sf0 <= GP_FLT_EPSILON)) {
                        step = dX_ * density_i;
                        h_int = dX_ / (e.grammage - Xi);
                } else {
                        /* Step length of a linear density profile
                         * (pumas.c:6676-6683). */
                        const double drho = density1 - density;
                        double tmp = GP_ADD(GP_MUL(density, density),
                            GP_MUL(GP_MUL(2., dX_), drho) / sf0);
                        tmp = (tmp > GP_FLT_EPSILON) ? sqrt(tmp) : 0;
                        h_int = GP_SUB(tmp, density) / drho;
                        step = GP_MUL(step, h_int);
                }
                e.grammage = grammage_max;
                if (!(event & GPUMAS_EVENT_LIMIT_ENERGY)) {
                        if (scheme <= GPUMAS_MODE_MIXED) {
                                if (scheme != GPUMAS_MODE_DISABLED)
                                        k1 = gp_cel_kinetic_energy(T, scheme,
                                            material,
                                            Xtot - sgn * (e.grammage - Xi));
                                event = e.step_foreseen;
                        } else if (!(event & (GPUMAS_EVENT_VERTEX_COULOMB |
                                                 GPUMAS_EVENT_VERTEX_DEL))) {
                                k1 = e.energy -
                                    sgn * (e.grammage - Xi) * dk / dX;
                                if (k1 < 0.) k1 = 0.;
                                event = GPUMAS_EVENT_LIMIT_GRAMMAGE;
                        }
                }
                const double ds_ = step - sf0;
                e.pos[0] = GP_ADD(e.pos[0], GP_MUL(ds_, sd0));
                e.pos[1] = GP_ADD(e.pos[1], GP_MUL(ds_, sd1));
                e.pos[2] = GP_ADD(e.pos[2], GP_MUL(ds_, sd2));
        }

        int decayed = 0;
        double time_max =
            (cfg.event & GPUMAS_EVENT_LIMIT_TIME) ? cfg.limit_time : 0.;
        if (cfg.decay == GPUMAS_MODE_RANDOMISED) {
                if ((time_max <= 0.) || (e.lifetime < time_max)) {
                        time_max = e.lifetime;
                        decayed = 1;
                }
        }
        const double sf1 = step;
        if (straight && (scheme != GPUMAS_MODE_DISABLED)) {
                const double Ti =
                    gp_cel_proper_time(T, scheme, material, e.energy);
                if (time_max > 0.) {
                        const double Tf =
                            Ti - sgn * (time_max - e.time) * density;
                        if (Tf > 0.) {
                                const double dxT = fabs(Xtot -
                                    gp_cel_grammage_as_time(
                                        T, scheme, material, Tf));
                                if (Xi + dxT < e.grammage) {
                                        event = GPUMAS_EVENT_LIMIT_TIME;
                                        e.time = time_max;
                                        e.decayed = decayed;
                                        step = dxT * density_i;
                                        if (step > sf1) step = sf1;
                                        e.grammage = Xi + dxT;
                                        const double xf = Xtot - sgn * dxT;
                                        k1 = gp_cel_kinetic_energy(
                                            T, scheme, material, xf);
                                }
                        }
                }
                if (event != GPUMAS_EVENT_LIMIT_TIME) {
                        const double Tf =
                            gp_cel_proper_time(T, scheme, material, k1);
                        /* Rounded as the reference's accumulation. */
                        e.time = GP_ADD(e.time,
                            GP_MUL(fabs(Tf - Ti), density_i));
                }
        } else {
                const double p_f =
                    (k1 <= 0) ? momentum : sqrt(k1 * (k1 + 2. * T.mass));
                const double ti = e.time;
                /* Correctly rounded reciprocals, products and sums: the
                 * time accumulates over the whole track, so it is rounded
                 * as the reference's expression is (pumas.c:6759-6760). */
                e.time = GP_ADD(e.time, GP_MUL(GP_MUL(GP_MUL(0.5, step),
                    T.mass), GP_ADD(__drcp_rn(momentum), __drcp_rn(p_f))));
                if ((time_max > 0.) && (e.time >= time_max)) {
                        event = GPUMAS_EVENT_LIMIT_TIME;
                        e.time = time_max;
                        e.decayed = decayed;
                        const double a = (momentum / p_f - 1.) / sf1;
                        const double c =
                            -2. * (time_max - ti) * momentum / T.mass;
                        if (a != 0.) {
                                double delta = GP_SUB(1., GP_MUL(a, c));
                                if (delta < 0.) delta = 0.;
                                step = 1. / a * (sqrt(delta) - 1.);
                        } else {
                                step = -0.5 * c;
                        }
                        if (step < 0.) step = 0.;
                        if (scheme != GPUMAS_MODE_DISABLED) {
                                const double p1 =
                                    momentum / GP_ADD(1, GP_MUL(a, step));
                                k1 = sqrt(GP_SUB(GP_MUL(p1, p1),
                                         GP_MUL(T.mass, T.mass))) - T.mass;
                                if (k1 < 0.) k1 = 0.;
                        }
                        const double Xf = Xi + dX;
                        if ((loc == NULL) || (density == density1))
                                e.grammage = Xi + step * density;
                        else
                                e.grammage = GP_ADD(Xi, GP_MUL(step,
                                    GP_ADD(density, GP_MUL(GP_MUL(0.5,
                                        step) / sf0, GP_SUB(density1,
                                        density)))));
                        if (e.grammage > Xf) e.grammage = Xf;
                }
        }
        if (event == GPUMAS_EVENT_LIMIT_TIME) {
                const double ds_ = step - sf1;
                e.pos[0] = GP_ADD(e.pos[0], GP_MUL(ds_, sd0));
                e.pos[1] = GP_ADD(e.pos[1], GP_MUL(ds_, sd1));
                e.pos[2] = GP_ADD(e.pos[2], GP_MUL(ds_, sd2));
        }

        e.step_event = event;
        e.energy = k1;
        e.distance += step;

        if (cfg.scattering == GPUMAS_MODE_MIXED) {
                if (e.energy <= 0.) {
                        e.step_invlb1 = invlb1;
                } else {
                        double mu0, invlb1_;
                        gp_table_get_msc(
                            T, scheme, material, e.energy, mu0, invlb1_);
                        e.step_invlb1 = density1 * invlb1_;
                }
        }
        if ((loc != NULL) && (rLarmor0 > 0. || loc->magnetized))
                gp_step_deflect(T, cfg, e, *loc, Bi, h_int, momentum, step,
                    rLarmor0, uT0);
        if ((invlb1 > 0.) || (e.step_invlb1 > 0.)) {
                double ilb1 = 0.25 * step * (invlb1 + e.step_invlb1);
                if (ilb1 > 1.) ilb1 = 1.;
                double mu;
                int trials = 0;
                do {
                        mu = -ilb1 * gp_log(gp_random(e));
                } while ((mu > 1.) && (++trials < cfg.max_trials));
                if (trials == cfg.max_trials)
                        e.status = GPUMAS_RETURN_INTERNAL_ERROR;
                gp_rotate(e, mu);
        }
        return out_medium;
}

/* Cap on the number of steps of one transport call; the reference has
 * none, the engine stops the event with an internal error instead. */
#define GP_MAX_STEPS 100000000

/* Loop carried locals of transport_with_stepping (pumas.c:5194-5514):
 * together with gp_event they are the whole state of an event between two
 * steps, which lets the stepping loop be suspended and resumed in another
 * kernel. */
struct gp_loop {
        int medium, material, straight, step_index;
        int new_medium;
        double density, ti, wi, Xi, Xf, dei, grammage_max, step_max_medium;
};

/* What an event needs next. */
enum gp_next {
        GP_NEXT_STEP = 1, /* another continuous step */
        GP_NEXT_DEL = 2,  /* a discrete energy loss (transport_do_del) */
        GP_NEXT_EHS = 3,  /* a hard elastic scatter (transport_do_ehs) */
        GP_NEXT_DONE = 4  /* the transport call is over */
};

/* Prologue of transport_with_stepping, up to the first transport_limit
 * (pumas.c:5201-5271). Returns GP_NEXT_STEP or GP_NEXT_DONE (then *event is
 * the end event). */
static __device__ __forceinline__ int gp_stepping_begin(const gp_tables & T, const gp_config & cfg,
    const gpumas_geometry & g, gp_event & e, gp_loop & L, int & event,
    gp_rec * rec = NULL, const gp_loc * loc = NULL)
{
        L.material = gp_medium_material(g, L.medium);
        const int scheme = cfg.energy_loss;
        L.straight = ((cfg.scattering == GPUMAS_MODE_DISABLED) &&
                         (scheme <= GPUMAS_MODE_MIXED) &&
                         ((loc == NULL) || ((loc->step_max <= 0.) &&
                                               !loc->magnetized))) ? 1 : 0;
        e.step_event = GPUMAS_EVENT_NONE;
        if (rec != NULL)
                gp_rec_frame(rec, e, L.medium, GPUMAS_EVENT_START);
        L.ti = e.time;
        L.wi = e.weight;
        L.Xi = e.grammage;
        if (scheme > GPUMAS_MODE_DISABLED) {
                L.Xf = gp_cel_grammage(T, scheme, L.material, e.energy);
                L.dei = 1. /
                    gp_cel_energy_loss(T, scheme, L.material, e.energy);
        } else {
                L.Xf = L.dei = 0.;
        }
        event = GPUMAS_EVENT_NONE;
        if ((cfg.event & GPUMAS_EVENT_LIMIT_DISTANCE) &&
            (e.distance >= cfg.limit_distance)) {
                event = GPUMAS_EVENT_LIMIT_DISTANCE;
                return GP_NEXT_DONE;
        }
        if ((cfg.event & GPUMAS_EVENT_LIMIT_GRAMMAGE) &&
            (e.grammage >= cfg.limit_grammage)) {
                event = GPUMAS_EVENT_LIMIT_GRAMMAGE;
                return GP_NEXT_DONE;
        }
        if ((cfg.event & GPUMAS_EVENT_LIMIT_TIME) &&
            (e.time >= cfg.limit_time)) {
                event = GPUMAS_EVENT_LIMIT_TIME;
                return GP_NEXT_DONE;
        }
        if (e.weight <= 0.) {
                event = GPUMAS_EVENT_WEIGHT;
                return GP_NEXT_DONE;
        }
        L.grammage_max = 0.;
        e.step_event = GPUMAS_EVENT_NONE;
        e.step_first = 1;
        e.step_X_limit = (cfg.event & GPUMAS_EVENT_LIMIT_ENERGY) ?
            gp_cel_grammage(T,
                (scheme > GPUMAS_MODE_DISABLED) ? scheme : GPUMAS_MODE_CSDA,
                L.material, cfg.limit_energy) :
            0.;
        e.step_invlb1 = 0;
        gp_limit(T, cfg, e, L.material, L.Xi, L.Xf, L.grammage_max);
        if (e.step_event) {
                event = e.step_event;
                return GP_NEXT_DONE;
        }
        L.step_index = 1;
        return GP_NEXT_STEP;
}

/* Refresh of the initial conditions and limits after an event
 * (pumas.c:5479-5488). */
static __device__ __forceinline__ int gp_stepping_relimit(const gp_tables & T, const gp_config & cfg,
    gp_event & e, gp_loop & L, int & event)
{
        L.ti = e.time;
        L.wi = e.weight;
        L.Xi = e.grammage;
        if (cfg.energy_loss >= GPUMAS_MODE_CSDA) {
                L.Xf = gp_cel_grammage(T, cfg.energy_loss, L.material,
                    e.energy);
                L.dei = 1. / gp_cel_energy_loss(T, cfg.energy_loss,
                                 L.material, e.energy);
        }
        gp_limit(T, cfg, e, L.material, L.Xi, L.Xf, L.grammage_max);
        if (e.step_event) {
                event = e.step_event;
                return GP_NEXT_DONE;
        }
        return GP_NEXT_STEP;
}

/* Update of non-uniform locals after a DEL or an EHS (pumas.c:5403-5414).
 * Returns GP_NEXT_DONE on a density error, else GP_NEXT_STEP. */
GPD int gp_stepping_locals(const gp_tables & T, const gp_config & cfg,
    gp_event & e, gp_loop & L, gp_loc * loc, int & event)
{
        if ((loc == NULL) || (loc->step_max <= 0.)) return GP_NEXT_STEP;
        loc->step_max = gp_set_locals(T, cfg, e, L.medium, L.density, *loc);
        loc->density = L.density;
        if (L.density <= 0.) {
                e.status = GPUMAS_RETURN_DENSITY_ERROR;
                event = e.step_event;
                return GP_NEXT_DONE;
        }
        return GP_NEXT_STEP;
}

/* Weight update at a stepping event (pumas.c:5309-5321): backward
 * Jacobian and decay weight since the last event. */
GPD void gp_stepping_weight(const gp_tables & T, const gp_config & cfg,
    gp_event & e, const gp_loop & L)
{
        if ((cfg.direction == GPUMAS_MODE_BACKWARD) &&
            (cfg.energy_loss >= GPUMAS_MODE_CSDA)) {
                const double wt = (cfg.decay == GPUMAS_MODE_WEIGHTED) ?
                    gp_exp(-fabs(e.time - L.ti) / T.ctau) : 1.;
                e.weight = L.wi * wt * L.dei *
                    gp_cel_energy_loss(T, cfg.energy_loss, L.material,
                        e.energy);
        } else if (cfg.decay == GPUMAS_MODE_WEIGHTED) {
                e.weight = L.wi * gp_exp(-fabs(e.time - L.ti) / T.ctau);
        }
}

/* One iteration of the stepping loop up to the dispatch of its event
 * (pumas.c:5277-5329 and the medium change of 5417-5467). */
static __device__ __forceinline__ int gp_stepping_step(const gp_tables & T, const gp_config & cfg,
    const gpumas_geometry & g, gp_event & e, gp_loop & L, int & event,
    gp_rec * rec = NULL, gp_loc * loc = NULL)
{
        if (L.step_index > 1) {
                const int m = gp_locate(g, e);
                L.step_max_medium = gp_step_proposal(cfg, g, e, m);
                if (L.step_max_medium > 0.)
                        L.step_max_medium += 0.5 * GP_STEP_MIN;
        }
        L.new_medium = gp_step(T, cfg, g, e, L.straight, L.medium,
            L.material, L.density, L.grammage_max, L.step_max_medium, loc);
        if (loc != NULL) L.density = loc->density;
        L.step_index++;
        if (e.status != GPUMAS_RETURN_SUCCESS) {
                event = e.step_event;
                return GP_NEXT_DONE;
        }
        if (L.step_index >= GP_MAX_STEPS) {
                e.status = GPUMAS_RETURN_INTERNAL_ERROR;
                event = e.step_event;
                return GP_NEXT_DONE;
        }
        /* A recorded step (every period-th, pumas.c:5296-5303) also updates
         * the weight; the update is idempotent until the next event. */
        const int record_step = (rec != NULL) && (rec->period > 0) &&
            (L.step_index != 1) && ((L.step_index % rec->period) == 0);
        if (!e.step_event && !record_step) return GP_NEXT_STEP;

        /* A DEL or an EHS leaves with its weight update still to be made
         * (gp_stepping_weight, first thing of the DEL and EHS phases): in
         * the pool engine it then runs in the compact DEL and EHS kernels
         * instead of a few lanes of each step warp. */
        if (!(e.step_event & (GPUMAS_EVENT_LIMIT | GPUMAS_EVENT_WEIGHT |
                                GPUMAS_EVENT_VERTEX_DECAY))) {
                if (e.step_event & GPUMAS_EVENT_VERTEX_DEL) return GP_NEXT_DEL;
                if (e.step_event & GPUMAS_EVENT_VERTEX_COULOMB)
                        return GP_NEXT_EHS;
        }
        const int scheme = cfg.energy_loss;
        gp_stepping_weight(T, cfg, e, L);

        if (!e.step_event) {
                gp_rec_frame(rec, e, L.medium, GPUMAS_EVENT_NONE);
                return GP_NEXT_STEP;
        }
        if (e.step_event & (GPUMAS_EVENT_LIMIT | GPUMAS_EVENT_WEIGHT |
                               GPUMAS_EVENT_VERTEX_DECAY)) {
                event = e.step_event;
                return GP_NEXT_DONE;
        } else if (e.step_event & GPUMAS_EVENT_MEDIUM) {
                L.medium = L.new_medium;
                if ((L.medium < 0) || (cfg.event & GPUMAS_EVENT_MEDIUM)) {
                        event = e.step_event;
                        return GP_NEXT_DONE;
                }
                L.material = gp_medium_material(g, L.medium);
                if (loc != NULL) {
                        loc->step_max = gp_set_locals(
                            T, cfg, e, L.medium, L.density, *loc);
                        loc->density = L.density;
                        L.straight =
                            ((cfg.scattering == GPUMAS_MODE_DISABLED) &&
                                (scheme <= GPUMAS_MODE_MIXED) &&
                                (loc->step_max <= 0.) && !loc->magnetized) ?
                            1 : 0;
                } else {
                        L.density = gp_medium_density(T, g, L.medium);
                }
                if (L.density <= 0.) {
                        e.status = GPUMAS_RETURN_DENSITY_ERROR;
                        event = e.step_event;
                        return GP_NEXT_DONE;
                }
                e.step_X_limit = (cfg.event & GPUMAS_EVENT_LIMIT_ENERGY) ?
                    gp_cel_grammage(T,
                        scheme > GPUMAS_MODE_DISABLED ? scheme :
                                                        GPUMAS_MODE_CSDA,
                        L.material, cfg.limit_energy) :
                    0.;
                e.step_first = 1;
                e.step_invlb1 = 0;
                if ((rec != NULL) && !(cfg.event & GPUMAS_EVENT_MEDIUM))
                        gp_rec_frame(rec, e, L.medium, e.step_event);
                return gp_stepping_relimit(T, cfg, e, L, event);
        }
        e.status = GPUMAS_RETURN_INTERNAL_ERROR;
        event = e.step_event;
        return GP_NEXT_DONE;
}

/* Tail of a DEL in the stepping loop, once the polar angle is applied
 * (pumas.c:5361-5374 and 5479-5488). */
static __device__ __forceinline__ int gp_stepping_del_end(const gp_tables & T,
    const gp_config & cfg, gp_event & e, gp_loop & L, int & event,
    gp_loc * loc = NULL)
{
        if ((cfg.event & e.step_event) ||
            (e.step_event == GPUMAS_EVENT_WEIGHT) ||
            (e.status != GPUMAS_RETURN_SUCCESS)) {
                event = e.step_event;
                return GP_NEXT_DONE;
        }
        e.step_first = 1;
        e.step_invlb1 = 0;
        if (gp_stepping_locals(T, cfg, e, L, loc, event) == GP_NEXT_DONE)
                return GP_NEXT_DONE;
        return gp_stepping_relimit(T, cfg, e, L, event);
}

/* DEL of the stepping loop (pumas.c:5336-5374 and 5479-5488). When
 * recording with a positive period, the pre step point (energy and
 * direction before the DEL, with the DEL flag) and, unless the transport
 * stops, the post step point are recorded. */
static __device__ __forceinline__ int gp_stepping_del(const gp_tables & T,
    const gp_config & cfg, gp_event & e, gp_loop & L, int & event,
    gp_rec * rec = NULL, gp_loc * loc = NULL)
{
        gp_stepping_weight(T, cfg, e, L);
        if ((rec == NULL) || (rec->period <= 0)) {
                gp_do_del(T, cfg, e, L.material);
                return gp_stepping_del_end(T, cfg, e, L, event, loc);
        }
        const double ki = e.energy;
        const double ui[3] = { e.dir[0], e.dir[1], e.dir[2] };
        gp_do_del(T, cfg, e, L.material);
        {
                const double kf = e.energy;
                const double uf[3] = { e.dir[0], e.dir[1], e.dir[2] };
                e.energy = ki;
                e.dir[0] = ui[0], e.dir[1] = ui[1], e.dir[2] = ui[2];
                gp_rec_frame(rec, e, L.medium, e.step_event);
                e.energy = kf;
                e.dir[0] = uf[0], e.dir[1] = uf[1], e.dir[2] = uf[2];
        }
        if ((cfg.event & e.step_event) ||
            (e.step_event == GPUMAS_EVENT_WEIGHT) ||
            (e.status != GPUMAS_RETURN_SUCCESS)) {
                event = e.step_event;
                return GP_NEXT_DONE;
        }
        gp_rec_frame(rec, e, L.medium, GPUMAS_EVENT_NONE);
        e.step_first = 1;
        e.step_invlb1 = 0;
        if (gp_stepping_locals(T, cfg, e, L, loc, event) == GP_NEXT_DONE)
                return GP_NEXT_DONE;
        return gp_stepping_relimit(T, cfg, e, L, event);
}

/* EHS of the stepping loop (pumas.c:5393-5400 and 5479-5488). */
static __device__ __forceinline__ int gp_stepping_ehs(const gp_tables & T, const gp_config & cfg,
    gp_event & e, gp_loop & L, int & event, gp_loc * loc = NULL)
{
        gp_stepping_weight(T, cfg, e, L);
        gp_do_ehs(T, cfg, e, L.material);
        if ((cfg.event & e.step_event) ||
            (e.status != GPUMAS_RETURN_SUCCESS)) {
                event = e.step_event;
                return GP_NEXT_DONE;
        }
        if (gp_stepping_locals(T, cfg, e, L, loc, event) == GP_NEXT_DONE)
                return GP_NEXT_DONE;
        return gp_stepping_relimit(T, cfg, e, L, event);
}

/* Epilogue: protection of the final kinetic energy (pumas.c:5491-5505). */
GPD void gp_stepping_end(const gp_config & cfg, gp_event & e)
{
        if (cfg.direction == GPUMAS_MODE_FORWARD) {
                const double kinetic_min =
                    (cfg.event & GPUMAS_EVENT_LIMIT_ENERGY) ?
                    cfg.limit_energy : 0.;
                if (fabs(e.energy - kinetic_min) < GP_FLT_EPSILON)
                        e.energy = kinetic_min;
        } else {
                if ((cfg.event & GPUMAS_EVENT_LIMIT_ENERGY) &&
                    (fabs(e.energy - cfg.limit_energy) < GP_FLT_EPSILON))
                        e.energy = cfg.limit_energy;
        }
}

/* Normalised magnetic rotation angle of the deterministic CEL, in
 * kg/m^2/T (cel_magnetic_rotation, pumas.c:3849-3883): the proper time
 * integral from the kinetic energy down to the table's bottom. */
GPD double gp_cel_magnetic_rotation(
    const gp_tables & T, int material, double kinetic)
{
        const int imax = T.n_energies - 1;
        const double factor = GP_LARMOR_FACTOR / T.mass;
        const double Tmax = __ldg(T.T + GP_ROW(0, material) + imax);
        if (kinetic <= __ldg(T.K)) return GP_MUL(Tmax, factor);
        if (kinetic >= __ldg(T.K + imax)) return 0.;
        const double t = gp_baked(T, GP_LUT_K, T.K,
            GP_C_T(T.n_materials, 0, material), kinetic);
        return GP_MUL(GP_SUB(Tmax, t), factor);
}

/* Magnetic transport moments x, y, z of the CSDA down from `kinetic` in a
 * uniform medium and transverse field (csda_magnetic_transport,
 * pumas.c:5095-5171): the tabulated moments of the 8 orders, combined with
 * the reference's polynomial fits of cos and sin over [0, 2 pi] (data of
 * the algorithm, kept as they are). Returns a pumas return code. */
GPD int gp_csda_magnetic_transport(const gp_tables & T, int material,
    double density, double magnet, double charge, double kinetic,
    double phase, double & x, double & y, double & z)
{
        const int imax = T.n_energies - 1;
        double k0 = kinetic;
        int i1, i2;
        if (kinetic <= __ldg(T.K)) {
                k0 = __ldg(T.K);
                i1 = 0;
                i2 = 1;
        } else if (kinetic >= __ldg(T.K + imax)) {
                y = 0.;
                x = z = -GP_SUB(gp_cel_grammage(T, GPUMAS_MODE_CSDA, material,
                                    kinetic),
                            __ldg(T.X + GP_ROW(0, material) + imax));
                return GPUMAS_RETURN_SUCCESS;
        } else {
                i1 = gp_index(T, GP_LUT_K, T.K, k0);
                i2 = i1 + 1;
        }
        if (fabs(phase) > 2.0 * GP_PI) return GPUMAS_RETURN_VALUE_ERROR;
        const double poly_x[8] = { 1.000000000e+000, 0.000000000e+000,
                -5.000000000e-001, -1.048969541e-002, 5.597396438e-002,
                -6.401353612e-003, -4.495849930e-004, 6.583532135e-005 };
        const double poly_y[8] = { 0.000000000e+000, 1.000000000e+000,
                -1.400755143e-002, -1.350173383e-001, -2.838778336e-002,
                2.123237056e-002, -3.094290091e-003, 1.409012754e-004 };
        const double a = GP_MUL(-magnet, charge) / density;
        const double * L = T.Li + (long)material * 8 * T.n_energies;
        double x1 = 0., x2 = 0., y1 = 0., y2 = 0., u = 1.;
        for (int j = 0; j < 8; j++) {
                const double l1 = __ldg(L + j * T.n_energies + i1);
                const double l2 = __ldg(L + j * T.n_energies + i2);
                const double ux = GP_MUL(u, poly_x[j]);
                const double uy = GP_MUL(u, poly_y[j]);
                x1 = GP_ADD(x1, GP_MUL(ux, l1));
                y1 = GP_ADD(y1, GP_MUL(uy, l1));
                x2 = GP_ADD(x2, GP_MUL(ux, l2));
                y2 = GP_ADD(y2, GP_MUL(uy, l2));
                u = GP_MUL(u, a);
        }
        const double z1 = __ldg(L + i1), z2 = __ldg(L + i2);
        const double K1 = __ldg(T.K + i1);
        const double h = GP_SUB(k0, K1) / GP_SUB(__ldg(T.K + i2), K1);
        x = GP_ADD(x1, GP_MUL(h, GP_SUB(x2, x1))) / density;
        y = GP_ADD(y1, GP_MUL(h, GP_SUB(y2, y1))) / density;
        z = GP_ADD(z1, GP_MUL(h, GP_SUB(z2, z1))) / density;
        return GPUMAS_RETURN_SUCCESS;
}

/* End point of a CSDA track of length `distance` from kinetic energy ki to
 * e.energy in a uniform medium and field (transport_csda_deflect,
 * pumas.c:4968-5075), in the field's frame: ez along the field, ex and ey
 * across it. Returns a pumas return code; as in the reference, the
 * position and direction stay as they are when the track has no rotation
 * at all or on an error. */
GPD int gp_csda_deflect(const gp_tables & T, gp_event & e, int material,
    double density, const double * m, double ki, double distance)
{
        const double charge = e.charge;
        const double kf = e.energy;
        const double * u = e.dir;
        const double b0 = sqrt(GP_ADD(GP_ADD(GP_MUL(m[0], m[0]),
            GP_MUL(m[1], m[1])), GP_MUL(m[2], m[2])));
        const double b0_i = 1.0 / b0;
        double ex[3], ey[3], ez[3];
        ey[0] = GP_MUL(GP_SUB(GP_MUL(u[2], m[1]), GP_MUL(u[1], m[2])), b0_i);
        ey[1] = GP_MUL(GP_SUB(GP_MUL(u[0], m[2]), GP_MUL(u[2], m[0])), b0_i);
        ey[2] = GP_MUL(GP_SUB(GP_MUL(u[1], m[0]), GP_MUL(u[0], m[1])), b0_i);
        const double d = GP_MUL(GP_MUL(b0_i, b0_i), GP_ADD(GP_ADD(
            GP_MUL(m[0], u[0]), GP_MUL(m[1], u[1])), GP_MUL(m[2], u[2])));
        for (int k = 0; k < 3; k++) {
                ez[k] = GP_MUL(m[k], d);
                ex[k] = GP_SUB(u[k], ez[k]);
        }
        const double a = GP_MUL(-b0, charge) / density;
        const double pi = GP_MUL(a, gp_cel_magnetic_rotation(T, material, ki));
        const double pf = GP_MUL(a, gp_cel_magnetic_rotation(T, material, kf));
        const double dp = GP_SUB(pf, pi);
        const double ps = fabs(GP_ADD(pi, pf));
        if (ps == 0.) return GPUMAS_RETURN_SUCCESS;
        const double dp0 = fabs(dp);
        double dx, dy, dz;
        if ((dp0 < 1E-02) && (dp0 / ps < 1E-02)) {
                /* Small rotation, linear in the distance. */
                dz = (ki >= kf) ? distance : -distance;
                const double sixth = 1 / 6.0;
                dx = GP_MUL(dz, GP_SUB(1.0, GP_MUL(GP_MUL(sixth, dp), dp)));
                dy = GP_MUL(GP_MUL(0.5, dz), dp);
        } else {
                double xi, yi, zi, xf, yf, zf;
                int rc = gp_csda_magnetic_transport(T, material, density, b0,
                    charge, ki, pi, xi, yi, zi);
                if (rc != GPUMAS_RETURN_SUCCESS) return rc;
                rc = gp_csda_magnetic_transport(T, material, density, b0,
                    charge, kf, pf, xf, yf, zf);
                if (rc != GPUMAS_RETURN_SUCCESS) return rc;
                const double si = sin(pi);
                const double ci = cos(pi);
                xf = GP_SUB(xf, xi);
                yf = GP_SUB(yf, yi);
                dx = GP_ADD(GP_MUL(ci, xf), GP_MUL(si, yf));
                dy = GP_ADD(GP_MUL(-si, xf), GP_MUL(ci, yf));
                dz = GP_SUB(zf, zi);
        }
        for (int k = 0; k < 3; k++)
                e.pos[k] = GP_ADD(e.pos[k], GP_ADD(GP_ADD(GP_MUL(dx, ex[k]),
                    GP_MUL(dy, ey[k])), GP_MUL(dz, ez[k])));
        const double s = sin(dp);
        const double c = cos(dp);
        for (int k = 0; k < 3; k++)
                e.dir[k] = GP_ADD(GP_ADD(GP_MUL(c, ex[k]), GP_MUL(s, ey[k])),
                    ez[k]);
        return GPUMAS_RETURN_SUCCESS;
}

/* transport_with_csda (pumas.c:4777-4949), with the deflection of a
 * uniform magnetic field when `magnet` is given. */
static __device__ __forceinline__ int gp_transport_csda(const gp_tables & T, const gp_config & cfg,
    gp_event & e, int material, double density, int medium = -1,
    gp_rec * rec = NULL, const double * magnet = NULL)
{
        const double ki = e.energy;
        const double di = e.distance;
        const double ti = e.time;
        const double xi = gp_cel_grammage(T, GPUMAS_MODE_CSDA, material, ki);
        const double Ti = gp_cel_proper_time(T, GPUMAS_MODE_CSDA, material, ki);
        int event = GPUMAS_EVENT_NONE;
        if (rec != NULL)
                gp_rec_frame(rec, e, medium, GPUMAS_EVENT_START);
        double xB;
        if (cfg.event & GPUMAS_EVENT_LIMIT_GRAMMAGE) {
                xB = cfg.limit_grammage - e.grammage;
                event = GPUMAS_EVENT_LIMIT_GRAMMAGE;
        } else
                xB = GP_DBL_MAX;
        if (cfg.event & GPUMAS_EVENT_LIMIT_DISTANCE) {
                const double xD = density * (cfg.limit_distance - di);
                if (xD < xB) {
                        xB = xD;
                        event = GPUMAS_EVENT_LIMIT_DISTANCE;
                }
        }
        int decayed = 0;
        double time_max =
            (cfg.event & GPUMAS_EVENT_LIMIT_TIME) ? cfg.limit_time : 0.;
        if (cfg.decay == GPUMAS_MODE_RANDOMISED) {
                if ((time_max <= 0.) || (e.lifetime < time_max)) {
                        time_max = e.lifetime;
                        decayed = 1;
                }
        }
        if (time_max > 0.) {
                const double dt = time_max - ti;
                if (dt <= 0.) {
                        xB = 0.;
                        event = GPUMAS_EVENT_LIMIT_TIME;
                } else {
                        const double sgn =
                            (cfg.direction == GPUMAS_MODE_FORWARD) ? 1. : -1.;
                        const double Tf = Ti - sgn * dt * density;
                        if (Tf > 0.) {
                                const double xT = fabs(xi -
                                    gp_cel_grammage_as_time(
                                        T, GPUMAS_MODE_CSDA, material, Tf));
                                if (xT < xB) {
                                        xB = xT;
                                        event = GPUMAS_EVENT_LIMIT_TIME;
                                }
                        }
                }
        }
        if (xB <= 0.) return event;
        double xf, kf;
        if (cfg.direction == GPUMAS_MODE_FORWARD) {
                if (xi > xB) {
                        xf = xi - xB;
                        if (xB < GP_EPSILON_X * xi) {
                                kf = ki - gp_cel_energy_loss(T,
                                    GPUMAS_MODE_CSDA, material, ki) * xB;
                                if (kf < 0.) kf = 0.;
                        } else {
                                kf = gp_cel_kinetic_energy(
                                    T, GPUMAS_MODE_CSDA, material, xf);
                        }
                } else {
                        xf = kf = 0.;
                        event = GPUMAS_EVENT_LIMIT_ENERGY;
                }
                if (cfg.event & GPUMAS_EVENT_LIMIT_ENERGY) {
                        if (ki <= cfg.limit_energy)
                                return GPUMAS_EVENT_LIMIT_ENERGY;
                        if (kf < cfg.limit_energy) {
                                kf = cfg.limit_energy;
                                xf = gp_cel_grammage(
                                    T, GPUMAS_MODE_CSDA, material, kf);
                                event = GPUMAS_EVENT_LIMIT_ENERGY;
                        }
                }
        } else {
                if (xB == GP_DBL_MAX) {
                        xf = xB;
                        kf = GP_DBL_MAX;
                } else {
                        xf = xB + xi;
                        if (xB < GP_EPSILON_X * xi) {
                                kf = ki + gp_cel_energy_loss(T,
                                    GPUMAS_MODE_CSDA, material, ki) * xB;
                        } else {
                                kf = gp_cel_kinetic_energy(
                                    T, GPUMAS_MODE_CSDA, material, xf);
                        }
                }
                if (cfg.event & GPUMAS_EVENT_LIMIT_ENERGY) {
                        if (ki >= cfg.limit_energy)
                                return GPUMAS_EVENT_LIMIT_ENERGY;
                        if (kf > cfg.limit_energy) {
                                kf = cfg.limit_energy;
                                xf = gp_cel_grammage(
                                    T, GPUMAS_MODE_CSDA, material, kf);
                                event = GPUMAS_EVENT_LIMIT_ENERGY;
                        }
                }
        }
        const double distance = fabs(xf - xi) / density;
        e.energy = kf;
        if (event == GPUMAS_EVENT_LIMIT_DISTANCE)
                e.distance = cfg.limit_distance;
        else
                e.distance += distance;
        if (event == GPUMAS_EVENT_LIMIT_GRAMMAGE)
                e.grammage = cfg.limit_grammage;
        else
                e.grammage += distance * density;
        if (event == GPUMAS_EVENT_LIMIT_TIME) {
                e.time = time_max;
                e.decayed = decayed;
                if (decayed) event = GPUMAS_EVENT_VERTEX_DECAY;
        } else
                e.time += fabs(Ti - gp_cel_proper_time(
                                        T, GPUMAS_MODE_CSDA, material, kf)) /
                    density;
        if (cfg.direction == GPUMAS_MODE_BACKWARD)
                e.weight *=
                    gp_cel_energy_loss(T, GPUMAS_MODE_CSDA, material, kf) /
                    gp_cel_energy_loss(T, GPUMAS_MODE_CSDA, material, ki);
        if (cfg.decay == GPUMAS_MODE_WEIGHTED)
                e.weight *= gp_exp(-fabs(ti - e.time) / T.ctau);
        if (magnet != NULL) {
                const int rc = gp_csda_deflect(
                    T, e, material, density, magnet, ki, distance);
                if (rc != GPUMAS_RETURN_SUCCESS) {
                        e.status = rc;
                        return event;
                }
        } else {
                const double path = (cfg.direction == GPUMAS_MODE_FORWARD) ?
                    distance : -distance;
                e.pos[0] += path * e.dir[0];
                e.pos[1] += path * e.dir[1];
                e.pos[2] += path * e.dir[2];
        }
        if (rec != NULL)
                gp_rec_frame(rec, e, medium, event | GPUMAS_EVENT_STOP);
        return event;
}

/* Continue an event's random stream at draw n, with the Box-Muller cache
 * of its previous call (the per context state that the reference keeps
 * between transport calls, pumas.c:426-477). */
GPD void gp_event_carry(gp_event & e, uint64_t n, int randn_done,
    double randn_next)
{
        e.n = (uint32_t)n;
        if (e.n & 1u) {
                uint32_t x[4];
                gp_philox(e.n >> 1, 0u, (uint32_t)e.id,
                    (uint32_t)(e.id >> 32), e.k0, e.k1, x);
                e.rnext = gp_word_to_uniform(x[2], x[3]);
        }
        e.randn_done = randn_done;
        e.randn_next = randn_next;
}

/* Prepare the event context for a new transport call. */
GPD void gp_event_init(gp_event & e, uint64_t seed, uint64_t id)
{
        e.step_first = 0;
        e.step_event = e.step_foreseen = 0;
        e.step_X_limit = e.step_invlb1 = 0.;
        e.randn_done = 0;
        e.randn_next = 0.;
        e.lifetime = 0.;
        e.id = id;
        e.n = 0;
        e.rnext = 0.;
        e.k0 = (uint32_t)seed;
        e.k1 = (uint32_t)(seed >> 32);
        e.steps = 0;
        e.status = GPUMAS_RETURN_SUCCESS;
}

/* Entry of pumas_context_transport (pumas.c:3114-3251) for one event, up
 * to the start of the stepping loop. The context level checks are done on
 * the host before the launch. Returns GP_NEXT_STEP, or GP_NEXT_DONE with
 * *event set (including the whole deterministic CSDA case). */
static __device__ __forceinline__ int gp_transport_begin(const gp_tables & T, const gp_config & cfg,
    const gpumas_geometry & g, gp_event & e, gp_loop & L, int & event,
    int & medium_in, gp_rec * rec = NULL, gp_loc * loc = NULL)
{
        event = GPUMAS_EVENT_NONE;
        medium_in = -1;
        L.medium = -1;
        if (e.decayed) {
                event = GPUMAS_EVENT_VERTEX_DECAY;
                return GP_NEXT_DONE;
        }
        {
                const double * const u = e.dir;
                const double norm2 = u[0] * u[0] + u[1] * u[1] + u[2] * u[2];
                if (fabs(norm2 - 1) > GP_FLT_EPSILON) {
                        e.status = GPUMAS_RETURN_DIRECTION_ERROR;
                        return GP_NEXT_DONE;
                }
        }
        const int medium = gp_locate(g, e);
        double step_max_medium = gp_step_proposal(cfg, g, e, medium);
        medium_in = medium;
        if (medium < 0) {
                event = GPUMAS_EVENT_MEDIUM;
                if (rec != NULL)
                        gp_rec_frame(rec, e, -1, GPUMAS_EVENT_MEDIUM |
                            GPUMAS_EVENT_START | GPUMAS_EVENT_STOP);
                return GP_NEXT_DONE;
        } else if (step_max_medium > 0.)
                step_max_medium += 0.5 * GP_STEP_MIN;
        if (loc != NULL) {
                loc->g = &g;
                loc->step_max = gp_set_locals(T, cfg, e, medium, L.density,
                    *loc);
                loc->density = L.density;
                if ((loc->step_max > 0.) && (loc->step_max < step_max_medium))
                        step_max_medium = loc->step_max;
        } else {
                L.density = gp_medium_density(T, g, medium);
        }
        if (L.density <= 0.) {
                e.status = GPUMAS_RETURN_DENSITY_ERROR;
                return GP_NEXT_DONE;
        }
        L.medium = medium;
        if (cfg.decay == GPUMAS_MODE_RANDOMISED) {
                const double u = gp_random(e);
                e.lifetime = e.time - T.ctau * gp_log(u);
        }
        int do_stepping = 1;
        if ((step_max_medium <= 0.) &&
            ((loc == NULL) || (loc->step_max <= 0.)) &&
            (cfg.energy_loss <= GPUMAS_MODE_CSDA)) {
                if ((cfg.energy_loss == GPUMAS_MODE_DISABLED) &&
                    ((cfg.event & GPUMAS_EVENT_LIMIT) == 0)) {
                        e.status = GPUMAS_RETURN_MISSING_LIMIT;
                        return GP_NEXT_DONE;
                } else if ((cfg.scattering == GPUMAS_MODE_DISABLED) &&
                    (cfg.energy_loss == GPUMAS_MODE_CSDA)) {
                        do_stepping = 0;
                }
        }
        if (!do_stepping) {
                event = gp_transport_csda(T, cfg, e,
                    gp_medium_material(g, medium), L.density, medium, rec,
                    ((loc != NULL) && loc->magnetized) ? loc->magnet : NULL);
                return GP_NEXT_DONE;
        }
        L.step_max_medium = step_max_medium;
        /* The early stops of the stepping prologue return as they are,
         * without the final energy protection (pumas.c:5250-5271). */
        return gp_stepping_begin(T, cfg, g, e, L, event, rec, loc);
}

/* Resume the stepping loop of an event at phase `next` and run it to its
 * end (the one thread per event form). */
static __device__ __forceinline__ void gp_transport_run(const gp_tables & T, const gp_config & cfg,
    const gpumas_geometry & g, gp_event & e, gp_loop & L, int next,
    int & event, gp_rec * rec = NULL, gp_loc * loc = NULL)
{
        while (next != GP_NEXT_DONE) {
                if (next == GP_NEXT_STEP)
                        next = gp_stepping_step(
                            T, cfg, g, e, L, event, rec, loc);
                else if (next == GP_NEXT_DEL)
                        next = gp_stepping_del(T, cfg, e, L, event, rec, loc);
                else
                        next = gp_stepping_ehs(T, cfg, e, L, event, loc);
        }
        gp_stepping_end(cfg, e);
        /* End of the track (pumas.c:5507-5510); a failed step returns
         * before it in the reference. */
        if ((rec != NULL) && (e.status == GPUMAS_RETURN_SUCCESS))
                gp_rec_frame(rec, e, L.medium,
                    e.step_event | GPUMAS_EVENT_STOP);
}

/* pumas_context_transport for one event, in one thread. */
static __device__ __forceinline__ void gp_transport(const gp_tables & T, const gp_config & cfg,
    const gpumas_geometry & g, gp_event & e, int & event, int & medium_in,
    int & medium_out, gp_rec * rec = NULL, gp_loc * loc = NULL)
{
        gp_loop L;
        const int next = gp_transport_begin(
            T, cfg, g, e, L, event, medium_in, rec, loc);
        if (next != GP_NEXT_DONE)
                gp_transport_run(T, cfg, g, e, L, next, event, rec, loc);
        medium_out = L.medium;
}

#endif /* GP_DEVICE_CUH */
