/*
 * gpumas_geometry.h -- device-side geometry descriptors for batched transport.
 *
 * The reference lets the user describe the geometry with a C callback,
 * `pumas_medium_cb` (pumas.h:477-511), which the transport calls in three
 * ways (pumas.c:3182, 5281, 6422):
 *   - (state, &medium, &step): locate the start medium and propose a step;
 *   - (state, NULL, &step):    propose the next geometric step;
 *   - (state, &medium, NULL):  locate the medium at the current position.
 * A host function pointer cannot run on the GPU, so this header replaces the
 * callback with plain descriptors whose locate/step functions are written once
 * as inline code that compiles both as C99 (host) and as CUDA (device). A host
 * medium callback built on these functions therefore proposes bit-identical
 * steps to the ones the GPU kernels use, which is what event-by-event parity
 * with a CPU run of the reference needs.
 *
 * Three kinds of geometry are provided:
 *   - GPUMAS_GEOMETRY_UNIFORM:   one medium filling all space (step 0, i.e.
 *                                "infinite" in the sense of pumas.h:489-493);
 *   - GPUMAS_GEOMETRY_SLABS:     a stack of horizontal slabs z in [z_i, z_i+1[,
 *                                vacuum (no medium) outside;
 *   - GPUMAS_GEOMETRY_HEIGHTMAP: a terrain z_s(x, y) given on a regular grid
 *                                and bilinearly interpolated, with one medium
 *                                below the surface and another one above it,
 *                                up to a ceiling z_top (vacuum above).
 *
 * Steps are always of PUMAS_STEP_CHECK type (pumas.h:461-475): the transport
 * adds half the minimum step and cross-checks boundary crossings.
 *
 * Arithmetic in this file is written without any fusable multiply-add chains
 * on the device (explicit __dmul_rn / __dadd_rn), so that host (gcc, no FMA
 * contraction) and device evaluate exactly the same roundings.
 */
#ifndef GPUMAS_GEOMETRY_H
#define GPUMAS_GEOMETRY_H

#ifdef __CUDACC__
#define GPUMAS_HD __host__ __device__ __forceinline__
#else
#define GPUMAS_HD static inline
#endif

#if defined(__CUDA_ARCH__)
#define GPUMAS_MUL(a, b) __dmul_rn((a), (b))
#define GPUMAS_ADD(a, b) __dadd_rn((a), (b))
#define GPUMAS_SUB(a, b) __dsub_rn((a), (b))
#else
#define GPUMAS_MUL(a, b) ((a) * (b))
#define GPUMAS_ADD(a, b) ((a) + (b))
#define GPUMAS_SUB(a, b) ((a) - (b))
#endif

#ifdef __cplusplus
extern "C" {
#endif

/** Geometry kinds. */
enum gpumas_geometry_kind {
        GPUMAS_GEOMETRY_UNIFORM = 0,
        GPUMAS_GEOMETRY_SLABS = 1,
        GPUMAS_GEOMETRY_HEIGHTMAP = 2
};

/**
 * A propagation medium: the material index in the physics tables and a
 * uniform density override in kg/m^3. A null or negative density selects the
 * material's default density. This is the device form of `struct
 * pumas_medium` (pumas.h:363-376) with a locals callback that returns a
 * constant density, no magnetic field and no step limit (pumas.c:5528-5552);
 * density profiles and fields are given by struct gpumas_locals.
 */
struct gpumas_medium {
        int material;
        double density;
};

/** Density models of struct gpumas_locals. */
enum gpumas_density_model {
        /** The medium's density (struct gpumas_medium), uniform. */
        GPUMAS_DENSITY_UNIFORM = 0,
        /** rho0 exp(-(axis . r - h0) / lambda), e.g. an isothermal
         * atmosphere with axis the local vertical. */
        GPUMAS_DENSITY_EXPONENTIAL = 1
};

/**
 * Local properties of a medium that vary in space or carry a magnetic
 * field: the device form of a `pumas_locals_cb` (pumas.h:324-349) that
 * fills `struct pumas_locals` (density and magnet, pumas.h:314-321).
 *
 * - GPUMAS_DENSITY_UNIFORM: the density of the medium entry, and a
 *   returned inhomogeneity size of 0 (a uniform medium).
 * - GPUMAS_DENSITY_EXPONENTIAL: density rho0 exp(-(axis . r - h0) /
 *   lambda) in kg/m^3 at position r, and a returned inhomogeneity size of
 *   lambda / max(|axis . u|, eps) for the direction u of the state, the
 *   projected attenuation length (the exponential atmosphere of the
 *   reference's examples/pumas/geometry.c:76-97).
 *
 * `magnet` is a uniform magnetic field in T (zero: no field). The
 * transport limits its steps to the inhomogeneity size times the context
 * accuracy (transport_set_locals, pumas.c:5528-5552). As in the reference,
 * the density and the field must be continuous inside a medium.
 */
struct gpumas_locals {
        int model;
        double rho0;
        double axis[3];
        double h0;
        double lambda;
        double eps;
        double magnet[3];
};

/** Minimum geometric step, in m (the reference's STEP_MIN, pumas.c:101). */
#define GPUMAS_STEP_MIN 1E-07

/**
 * A geometry descriptor. Array members point to host memory when the
 * descriptor is passed to the library (it copies them to the device); the
 * library's device copy has the same layout with device pointers.
 */
struct gpumas_geometry {
        int kind;
        /* Media referenced by the regions below. */
        int n_media;
        const struct gpumas_medium * media;

        /* GPUMAS_GEOMETRY_UNIFORM: the medium index filling all space. */
        int uniform_medium;

        /* GPUMAS_GEOMETRY_SLABS: n_slabs layers, slab_z holds the n_slabs + 1
         * increasing boundaries and slab_medium the medium of each layer. */
        int n_slabs;
        const double * slab_z;
        const int * slab_medium;

        /* GPUMAS_GEOMETRY_HEIGHTMAP: hm_nx x hm_ny nodes, node (i, j) sits at
         * (hm_x0 + i hm_dx, hm_y0 + j hm_dy) with height hm_z[j hm_nx + i].
         * Outside of the grid footprint there is no terrain (medium above
         * only). Above hm_ztop there is no medium. */
        int hm_nx, hm_ny;
        double hm_x0, hm_y0, hm_dx, hm_dy;
        const double * hm_z;
        int hm_below, hm_above;
        double hm_ztop;

        /* Local properties, NULL or one entry per medium. With NULL every
         * medium is uniform, at its density, without magnetic field. */
        const struct gpumas_locals * locals;
};

/* Slabs: index of the layer containing z, or -1 outside of the stack. */
GPUMAS_HD int gpumas_slab_layer(const struct gpumas_geometry * g, double z)
{
        const int n = g->n_slabs;
        if ((z < g->slab_z[0]) || (z >= g->slab_z[n])) return -1;
        int lo = 0, hi = n;
        while (hi - lo > 1) {
                const int mid = (lo + hi) / 2;
                if (z >= g->slab_z[mid])
                        lo = mid;
                else
                        hi = mid;
        }
        return lo;
}

/* Heightmap: surface height at (x, y) inside the footprint. */
GPUMAS_HD double gpumas_hm_height(
    const struct gpumas_geometry * g, int i, int j, double s, double r)
{
        const double * h = g->hm_z + j * g->hm_nx + i;
        const double h00 = h[0], h10 = h[1];
        const double h01 = h[g->hm_nx], h11 = h[g->hm_nx + 1];
        const double a = GPUMAS_ADD(h00, GPUMAS_MUL(s, GPUMAS_SUB(h10, h00)));
        const double b = GPUMAS_ADD(h01, GPUMAS_MUL(s, GPUMAS_SUB(h11, h01)));
        return GPUMAS_ADD(a, GPUMAS_MUL(r, GPUMAS_SUB(b, a)));
}

/* Heightmap: cell indices and reduced coordinates, or 0 if outside. */
GPUMAS_HD int gpumas_hm_cell(const struct gpumas_geometry * g, double x,
    double y, int * i, int * j, double * s, double * r)
{
        const double fx = (x - g->hm_x0) / g->hm_dx;
        const double fy = (y - g->hm_y0) / g->hm_dy;
        if ((fx < 0.) || (fy < 0.) || (fx >= (double)(g->hm_nx - 1)) ||
            (fy >= (double)(g->hm_ny - 1)))
                return 0;
        *i = (int)fx;
        *j = (int)fy;
        *s = fx - (double)(*i);
        *r = fy - (double)(*j);
        return 1;
}

/**
 * Locate the medium index at position r, or -1 if there is no medium.
 */
GPUMAS_HD int gpumas_geometry_locate(
    const struct gpumas_geometry * g, const double * r)
{
        if (g->kind == GPUMAS_GEOMETRY_UNIFORM) {
                return g->uniform_medium;
        } else if (g->kind == GPUMAS_GEOMETRY_SLABS) {
                const int layer = gpumas_slab_layer(g, r[2]);
                return (layer < 0) ? -1 : g->slab_medium[layer];
        } else {
                if (r[2] >= g->hm_ztop) return -1;
                int i, j;
                double s, t;
                if (!gpumas_hm_cell(g, r[0], r[1], &i, &j, &s, &t))
                        return g->hm_above;
                const double zs = gpumas_hm_height(g, i, j, s, t);
                return (r[2] < zs) ? g->hm_below : g->hm_above;
        }
}

/* Exponent of an exponential density model at position r,
 * -(axis . r - h0) / lambda. */
GPUMAS_HD double gpumas_locals_exponent(
    const struct gpumas_locals * l, const double * r)
{
        const double s = GPUMAS_ADD(GPUMAS_ADD(GPUMAS_MUL(l->axis[0], r[0]),
            GPUMAS_MUL(l->axis[1], r[1])), GPUMAS_MUL(l->axis[2], r[2]));
        return -GPUMAS_SUB(s, l->h0) / l->lambda;
}

/* Inhomogeneity size of an exponential density model for the state
 * direction u, lambda / max(|axis . u|, eps). */
GPUMAS_HD double gpumas_locals_size(
    const struct gpumas_locals * l, const double * u)
{
        double c = fabs(GPUMAS_ADD(GPUMAS_ADD(GPUMAS_MUL(l->axis[0], u[0]),
            GPUMAS_MUL(l->axis[1], u[1])), GPUMAS_MUL(l->axis[2], u[2])));
        if (c <= l->eps) c = l->eps;
        return l->lambda / c;
}

/* Smallest root in ]0, tmax] of c0 + c1 t + c2 t^2, or -1 if none. */
GPUMAS_HD double gpumas_first_root(double c0, double c1, double c2,
    double tmax)
{
        double t = -1.;
        if (c2 == 0.) {
                if (c1 != 0.) {
                        const double t0 = -c0 / c1;
                        if ((t0 > 0.) && (t0 <= tmax)) t = t0;
                }
                return t;
        }
        const double delta = GPUMAS_SUB(GPUMAS_MUL(c1, c1),
            GPUMAS_MUL(4., GPUMAS_MUL(c0, c2)));
        if (delta < 0.) return -1.;
        const double sq = sqrt(delta);
        /* Numerically stable pair of roots. */
        const double qq = (c1 >= 0.) ? -0.5 * GPUMAS_ADD(c1, sq) :
                                       -0.5 * GPUMAS_SUB(c1, sq);
        double t1 = (qq != 0.) ? c0 / qq : -1.;
        double t2 = qq / c2;
        if (t1 > t2) {
                const double tmp = t1;
                t1 = t2;
                t2 = tmp;
        }
        if ((t1 > 0.) && (t1 <= tmax)) return t1;
        if ((t2 > 0.) && (t2 <= tmax)) return t2;
        return -1.;
}

/**
 * Propose a geometric step, in m, from position r along the unit direction
 * of motion u (which is minus the momentum direction in backward transport),
 * inside the medium of index `medium`. A null value means that there is no
 * geometric limit. The returned step is the distance to the next boundary
 * of the current region (or to the next heightmap cell edge), or the minimum
 * step if that distance rounds to zero.
 */
GPUMAS_HD double gpumas_geometry_step(const struct gpumas_geometry * g,
    const double * r, const double * u, int medium)
{
        if ((medium < 0) || (g->kind == GPUMAS_GEOMETRY_UNIFORM)) return 0.;

        if (g->kind == GPUMAS_GEOMETRY_SLABS) {
                const int layer = gpumas_slab_layer(g, r[2]);
                if (layer < 0) return 0.;
                double step;
                if (u[2] > 0.)
                        step = (g->slab_z[layer + 1] - r[2]) / u[2];
                else if (u[2] < 0.)
                        step = (g->slab_z[layer] - r[2]) / u[2];
                else
                        return 0.;
                return (step > 0.) ? step : GPUMAS_STEP_MIN;
        }

        /* Heightmap terrain. Distance to the ceiling first. */
        double step = 0.;
        if (u[2] > 0.) step = (g->hm_ztop - r[2]) / u[2];

        int i, j;
        double s, t;
        if (!gpumas_hm_cell(g, r[0], r[1], &i, &j, &s, &t)) {
                /* Outside of the footprint: distance to re-enter it. */
                const double xmax = GPUMAS_ADD(g->hm_x0,
                    GPUMAS_MUL((double)(g->hm_nx - 1), g->hm_dx));
                const double ymax = GPUMAS_ADD(g->hm_y0,
                    GPUMAS_MUL((double)(g->hm_ny - 1), g->hm_dy));
                double tin = 0.;
                int k;
                for (k = 0; k < 2; k++) {
                        const double lo = (k == 0) ? g->hm_x0 : g->hm_y0;
                        const double hi = (k == 0) ? xmax : ymax;
                        const double p = r[k], v = u[k];
                        double tk = 0.;
                        if ((p < lo) && (v > 0.))
                                tk = (lo - p) / v;
                        else if ((p >= hi) && (v < 0.))
                                tk = (hi - p) / v;
                        if (tk > tin) tin = tk;
                }
                if ((tin > 0.) && ((step <= 0.) || (tin < step))) step = tin;
                return (step > 0.) ? step : 0.;
        }

        /* Distance to the edges of the current cell. */
        double texit = -1.;
        int k;
        for (k = 0; k < 2; k++) {
                const double v = u[k] / ((k == 0) ? g->hm_dx : g->hm_dy);
                const double f = (k == 0) ? s : t;
                double tk = -1.;
                if (v > 0.)
                        tk = (1. - f) / v;
                else if (v < 0.)
                        tk = -f / v;
                if ((tk >= 0.) && ((texit < 0.) || (tk < texit))) texit = tk;
        }

        /* Crossing of the bilinear surface inside the cell. Along the ray
         * the surface height is quadratic in the path length. */
        const double * h = g->hm_z + j * g->hm_nx + i;
        const double h00 = h[0], h10 = h[1];
        const double h01 = h[g->hm_nx], h11 = h[g->hm_nx + 1];
        const double b = GPUMAS_SUB(h10, h00);
        const double c = GPUMAS_SUB(h01, h00);
        const double d = GPUMAS_ADD(GPUMAS_SUB(h00, h10),
            GPUMAS_SUB(h11, h01));
        const double ds = u[0] / g->hm_dx, dr = u[1] / g->hm_dy;
        const double zs = gpumas_hm_height(g, i, j, s, t);
        const double c0 = GPUMAS_SUB(r[2], zs);
        const double c1 = GPUMAS_SUB(GPUMAS_SUB(u[2],
            GPUMAS_ADD(GPUMAS_MUL(b, ds), GPUMAS_MUL(c, dr))),
            GPUMAS_MUL(d, GPUMAS_ADD(GPUMAS_MUL(s, dr), GPUMAS_MUL(t, ds))));
        const double c2 = -GPUMAS_MUL(d, GPUMAS_MUL(ds, dr));
        const double tmax = (texit >= 0.) ? texit : 1E+09;
        const double troot = gpumas_first_root(c0, c1, c2, tmax);

        double tgeo = (troot > 0.) ? troot : texit;
        if (tgeo >= 0.) {
                if (tgeo <= 0.) tgeo = GPUMAS_STEP_MIN;
                if ((step <= 0.) || (tgeo < step)) step = tgeo;
        }
        return step;
}

#ifdef __cplusplus
}
#endif
#endif /* GPUMAS_GEOMETRY_H */
