/*
 * straight_gpumas.c -- a C99 program using the engine through
 * include/gpumas.h only, shaped like the reference's example
 * examples/pumas/straight.c:133-179: muons transported backward with
 * straggled energy loss and no scattering through a given thickness of
 * standard rock (an infinite uniform medium with a distance limit), from a
 * detector at an elevation angle, kinetic energy log-uniform in
 * [energy_min, energy_max] with the Monte Carlo weight 1 / pdf, random
 * charge.
 *
 * The example's per event loop of pumas_context_transport becomes one call
 * of gpumas_context_transport over all events. The initial states come from
 * the engine's own Philox stream (gpumas_random_fill, domain 1) so that the
 * test can rebuild them. The program writes the initial and final states
 * (struct gpumas_state records) and the results to OUTPUT and prints the
 * mean weight.
 *
 * usage: straight_gpumas DUMP OUTPUT ROCK_THICKNESS ELEVATION EMIN EMAX N
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "gpumas.h"

/* Not defined by a strict C99 <math.h>. */
#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

static void * read_file(const char * path, size_t * size)
{
        FILE * f = fopen(path, "rb");
        if (f == NULL) return NULL;
        fseek(f, 0, SEEK_END);
        const long n = ftell(f);
        fseek(f, 0, SEEK_SET);
        void * data = malloc(n > 0 ? n : 1);
        if ((data != NULL) && (fread(data, 1, n, f) != (size_t)n)) {
                free(data);
                data = NULL;
        }
        fclose(f);
        *size = (size_t)n;
        return data;
}

static int check(int rc, const char * what)
{
        if (rc != GPUMAS_RETURN_SUCCESS)
                fprintf(stderr, "straight_gpumas: %s returned %d\n", what, rc);
        return rc;
}

int main(int narg, char * argv[])
{
        if (narg < 8) {
                fprintf(stderr, "usage: %s DUMP OUTPUT ROCK_THICKNESS "
                                "ELEVATION EMIN EMAX N\n", argv[0]);
                return EXIT_FAILURE;
        }
        const double rock_thickness = strtod(argv[3], NULL);
        const double elevation = strtod(argv[4], NULL);
        const double energy_min = strtod(argv[5], NULL);
        const double energy_max = strtod(argv[6], NULL);
        const int n = atoi(argv[7]);

        /* Physics: the bytes of a pumas_physics_dump stream. */
        size_t size = 0;
        void * dump = read_file(argv[1], &size);
        if (dump == NULL) {
                perror(argv[1]);
                return EXIT_FAILURE;
        }
        struct gpumas_physics * physics = NULL;
        if (check(gpumas_physics_load(&physics, dump, size),
                "gpumas_physics_load"))
                return EXIT_FAILURE;
        free(dump);

        /* The medium: infinite standard rock (the example's medium1). */
        int rock;
        if (check(gpumas_physics_material_index(physics, "StandardRock",
                      &rock), "gpumas_physics_material_index"))
                return EXIT_FAILURE;
        struct gpumas_medium media[1] = { { rock, 0. } };
        struct gpumas_geometry geometry;
        memset(&geometry, 0, sizeof(geometry));
        geometry.kind = GPUMAS_GEOMETRY_UNIFORM;
        geometry.n_media = 1;
        geometry.media = media;
        geometry.uniform_medium = 0;

        /* The context: straggled backward transport without scattering,
         * stopped at the rock depth. */
        struct gpumas_context * context = NULL;
        if (check(gpumas_context_create(&context, physics, 0),
                "gpumas_context_create"))
                return EXIT_FAILURE;
        context->mode.energy_loss = GPUMAS_MODE_STRAGGLED;
        context->mode.direction = GPUMAS_MODE_BACKWARD;
        context->mode.scattering = GPUMAS_MODE_DISABLED;
        context->limit.distance =
            (rock_thickness <= 0.) ? 1E-06 : rock_thickness;
        context->event |= GPUMAS_EVENT_LIMIT_DISTANCE;
        const uint64_t seed = 20240607;
        if (check(gpumas_context_random_seed_set(context, &seed),
                "gpumas_context_random_seed_set") ||
            check(gpumas_context_geometry_set(context, &geometry),
                "gpumas_context_geometry_set"))
                return EXIT_FAILURE;

        /* The final states at the detector: two uniform draws per event
         * from the Philox stream of (seed, domain 1, event 0). */
        double * u = malloc(2 * (size_t)n * sizeof(*u));
        struct gpumas_state * states = calloc(n, sizeof(*states));
        struct gpumas_state * initial = malloc(n * sizeof(*initial));
        struct gpumas_result * results = calloc(n, sizeof(*results));
        if ((u == NULL) || (states == NULL) || (initial == NULL) ||
            (results == NULL))
                return EXIT_FAILURE;
        if (check(gpumas_random_fill(seed, 1, 0, 0, 2 * (size_t)n, u),
                "gpumas_random_fill"))
                return EXIT_FAILURE;
        const double cos_theta = cos((90. - elevation) / 180. * M_PI);
        const double sin_theta = sqrt(1. - cos_theta * cos_theta);
        const double rk = log(energy_max / energy_min);
        int i;
        for (i = 0; i < n; i++) {
                double kf, wf;
                if (rk) {
                        kf = energy_min * exp(rk * u[2 * i]);
                        wf = kf * rk;
                } else {
                        kf = energy_min;
                        wf = 1;
                }
                states[i].charge = (u[2 * i + 1] > 0.5) ? 1 : -1;
                states[i].energy = kf;
                states[i].weight = 2 * wf;
                states[i].direction[0] = -sin_theta;
                states[i].direction[2] = -cos_theta;
        }
        memcpy(initial, states, n * sizeof(*states));

        /* Transport the muons backwards: one call for all of them. */
        const int rc = gpumas_context_transport(context, n, states, results, 0);
        if (check(rc, "gpumas_context_transport")) return EXIT_FAILURE;

        double w = 0.;
        for (i = 0; i < n; i++) w += states[i].weight;
        printf("mean weight %.17g\n", w / n);

        FILE * out = fopen(argv[2], "wb");
        if ((out == NULL) ||
            (fwrite(initial, sizeof(*initial), n, out) != (size_t)n) ||
            (fwrite(states, sizeof(*states), n, out) != (size_t)n) ||
            (fwrite(results, sizeof(*results), n, out) != (size_t)n)) {
                perror(argv[2]);
                return EXIT_FAILURE;
        }
        fclose(out);

        gpumas_context_destroy(&context);
        gpumas_physics_destroy(&physics);
        free(u);
        free(states);
        free(initial);
        free(results);
        return EXIT_SUCCESS;
}
