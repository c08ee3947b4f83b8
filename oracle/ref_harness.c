/*
 * ref_harness.c -- drives the unmodified reference library as an oracle.
 *
 * Test infrastructure only. This translation unit includes the reference's
 * own src/pumas.c (compiled from its source tree by oracle/Makefile, never
 * copied) so that the per-context Box-Muller cache of the reference
 * (`struct simulation_context`, pumas.c:426-477) can be reset between events.
 * Each event then starts from the same state as with a freshly created
 * context (pumas.c:2607-2609), which is what the GPU engine does.
 *
 * Random numbers come from the Philox stream of philox.h, keyed by
 * (seed, event id); geometry comes from gpumas_geometry.h. Events are
 * processed independently, optionally over OpenMP threads with one context
 * per thread, as the reference's threading model prescribes
 * (pumas.h:596-635).
 */
#include "pumas.c"

#include <stdint.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "gp_math.cuh"
#include "oracle.h"
#include "philox.h"

/* The loaded physics shared by all calls. */
static struct pumas_physics * ref_physics = NULL;

/* A medium with an optional uniform density override and optional local
 * properties (struct gpumas_locals). */
struct ref_medium {
        struct pumas_medium api;
        double density;
        const struct gpumas_locals * loc;
};

/* Per event data stored in the context's user memory. */
struct ref_event {
        struct oracle_stream stream;
        const struct gpumas_geometry * geometry;
        struct ref_medium * media;
        int steps;
};

/* The locals callback of a medium: a uniform density override, or the
 * density profile and field of its gpumas_locals, evaluated with the same
 * arithmetic as the device (gp_exp of gp_math.cuh). */
static double ref_locals(struct pumas_medium * medium,
    struct pumas_state * state, struct pumas_locals * locals)
{
        const struct ref_medium * m = (const struct ref_medium *)medium;
        const struct gpumas_locals * l = m->loc;
        locals->density = m->density;
        if (l == NULL) return 0.;
        memcpy(locals->magnet, l->magnet, sizeof(locals->magnet));
        if (l->model != GPUMAS_DENSITY_EXPONENTIAL) return 0.;
        locals->density =
            l->rho0 * gp_exp(gpumas_locals_exponent(l, state->position));
        return gpumas_locals_size(l, state->direction);
}

static enum pumas_step ref_medium_cb(struct pumas_context * context,
    struct pumas_state * state, struct pumas_medium ** medium_ptr,
    double * step_ptr)
{
        struct ref_event * data = context->user_data;
        const int m = gpumas_geometry_locate(data->geometry, state->position);
        if (medium_ptr != NULL)
                *medium_ptr = (m < 0) ? NULL : &data->media[m].api;
        if (step_ptr != NULL) {
                const double sgn =
                    (context->mode.direction == PUMAS_MODE_FORWARD) ? 1. : -1.;
                const double u[3] = { sgn * state->direction[0],
                        sgn * state->direction[1], sgn * state->direction[2] };
                *step_ptr = gpumas_geometry_step(
                    data->geometry, state->position, u, m);
                data->steps++;
        }
        return PUMAS_STEP_CHECK;
}

static double ref_random(struct pumas_context * context)
{
        struct ref_event * data = context->user_data;
        return oracle_stream_draw(&data->stream);
}

/* Create the physics from a MDF and dump it. */
int oracle_ref_physics_create(
    const char * mdf, const char * dedx, const char * dump_path)
{
        pumas_error_handler_set(NULL);
        struct pumas_physics * physics = NULL;
        enum pumas_return rc = pumas_physics_create(
            &physics, PUMAS_PARTICLE_MUON, mdf, dedx, NULL);
        if (rc != PUMAS_RETURN_SUCCESS) return rc;
        FILE * stream = fopen(dump_path, "wb");
        if (stream == NULL) {
                pumas_physics_destroy(&physics);
                return PUMAS_RETURN_PATH_ERROR;
        }
        rc = pumas_physics_dump(physics, stream);
        fclose(stream);
        pumas_physics_destroy(&physics);
        return rc;
}

/* Load a physics dump as the oracle's physics. */
int oracle_ref_load(const char * dump_path)
{
        pumas_error_handler_set(NULL);
        if (ref_physics != NULL) pumas_physics_destroy(&ref_physics);
        FILE * stream = fopen(dump_path, "rb");
        if (stream == NULL) return PUMAS_RETURN_PATH_ERROR;
        const enum pumas_return rc = pumas_physics_load(&ref_physics, stream);
        fclose(stream);
        return rc;
}

int oracle_ref_material_index(const char * name, int * index)
{
        if (ref_physics == NULL) return PUMAS_RETURN_PHYSICS_ERROR;
        return pumas_physics_material_index(ref_physics, name, index);
}

/* Tabulated properties, for known answer tests (pumas.h property API). */
int oracle_ref_property(int property, int scheme, int material,
    double kinetic, double * value)
{
        if (ref_physics == NULL) return PUMAS_RETURN_PHYSICS_ERROR;
        switch (property) {
        case 0:
                return pumas_physics_property_range(
                    ref_physics, scheme, material, kinetic, value);
        case 1:
                return pumas_physics_property_proper_time(
                    ref_physics, scheme, material, kinetic, value);
        case 2:
                return pumas_physics_property_kinetic_energy(
                    ref_physics, scheme, material, kinetic, value);
        case 3:
                return pumas_physics_property_stopping_power(
                    ref_physics, scheme, material, kinetic, value);
        case 4:
                return pumas_physics_property_energy_straggling(
                    ref_physics, material, kinetic, value);
        case 5:
                return pumas_physics_property_elastic_cutoff_angle(
                    ref_physics, material, kinetic, value);
        case 6:
                return pumas_physics_property_elastic_path(
                    ref_physics, material, kinetic, value);
        case 7:
                return pumas_physics_property_transport_path(
                    ref_physics, scheme, material, kinetic, value);
        case 8:
                return pumas_physics_property_cross_section(
                    ref_physics, material, kinetic, value);
        default:
                return PUMAS_RETURN_INDEX_ERROR;
        }
}

int oracle_ref_max_threads(void)
{
#ifdef _OPENMP
        return omp_get_max_threads();
#else
        return 1;
#endif
}

/* Transport a batch of events, one transport call per event. */
int oracle_ref_transport(const struct oracle_config * cfg,
    const struct gpumas_geometry * geometry, int64_t n, uint64_t first_event,
    struct oracle_state * states, struct oracle_result * results,
    int n_threads)
{
        if (ref_physics == NULL) return PUMAS_RETURN_PHYSICS_ERROR;
        pumas_error_handler_set(NULL);

        struct ref_medium * media =
            calloc(geometry->n_media > 0 ? geometry->n_media : 1,
                sizeof(*media));
        if (media == NULL) return PUMAS_RETURN_MEMORY_ERROR;
        int i;
        for (i = 0; i < geometry->n_media; i++) {
                media[i].api.material = geometry->media[i].material;
                media[i].density = geometry->media[i].density;
                media[i].loc = (geometry->locals != NULL) ?
                    geometry->locals + i : NULL;
                media[i].api.locals =
                    ((media[i].density > 0.) || (media[i].loc != NULL)) ?
                    &ref_locals : NULL;
        }

        int rc_all = PUMAS_RETURN_SUCCESS;
#ifdef _OPENMP
        if (n_threads <= 0) n_threads = omp_get_max_threads();
#pragma omp parallel num_threads(n_threads)
#endif
        {
                struct pumas_context * context = NULL;
                const int rc = pumas_context_create(
                    &context, ref_physics, sizeof(struct ref_event));
                if (rc != PUMAS_RETURN_SUCCESS) {
#ifdef _OPENMP
#pragma omp atomic write
#endif
                        rc_all = rc;
                } else {
                        context->medium = &ref_medium_cb;
                        context->random = &ref_random;
                        context->mode.energy_loss = cfg->energy_loss;
                        context->mode.decay = cfg->decay;
                        context->mode.direction = cfg->direction;
                        context->mode.scattering = cfg->scattering;
                        context->event = cfg->event;
                        context->limit.energy = cfg->limit_energy;
                        context->limit.distance = cfg->limit_distance;
                        context->limit.grammage = cfg->limit_grammage;
                        context->limit.time = cfg->limit_time;
                        context->accuracy = cfg->accuracy;
                        struct ref_event * data = context->user_data;
                        data->geometry = geometry;
                        data->media = media;
                        struct simulation_context * context_ =
                            (struct simulation_context *)context;
                        int64_t k;
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 256)
#endif
                        for (k = 0; k < n; k++) {
                                struct oracle_result * r = results + k;
                                data->stream.seed = cfg->seed;
                                data->stream.event = first_event + k;
                                data->stream.n = 0;
                                data->stream.next = 0.;
                                data->steps = 0;
                                context_->randn_done = 0;
                                context_->randn_next = 0.;
                                if (cfg->carry) {
                                        /* The event's own context as a
                                         * previous call left it. */
                                        oracle_stream_seek(
                                            &data->stream, r->draws);
                                        context_->randn_done = r->randn_done;
                                        context_->randn_next = r->randn_next;
                                }

                                enum pumas_event event = PUMAS_EVENT_NONE;
                                struct pumas_medium * m[2] = { NULL, NULL };
                                struct pumas_state * s =
                                    (struct pumas_state *)(states + k);
                                const enum pumas_return rck =
                                    pumas_context_transport(
                                        context, s, &event, m);
                                r->event = event;
                                r->medium_in = (m[0] == NULL) ? -1 :
                                    (int)((struct ref_medium *)m[0] - media);
                                r->medium_out = (m[1] == NULL) ? -1 :
                                    (int)((struct ref_medium *)m[1] - media);
                                r->status = rck;
                                r->steps = data->steps;
                                r->randn_done = context_->randn_done;
                                r->draws = data->stream.n;
                                r->randn_next = context_->randn_next;
                        }
                        pumas_context_destroy(&context);
                }
        }
        free(media);
        return rc_all;
}

/* Transport a batch of events with the reference's frame recorder
 * (pumas_recorder_create, default in-memory recording, pumas.c:2797-2852,
 * 7738-7780), one event after the other: event k's frames are copied to
 * frames[k * max_frames ...] (at most max_frames) and the recorder's frame
 * count to length[k]. */
int oracle_ref_transport_record(const struct oracle_config * cfg,
    const struct gpumas_geometry * geometry, int64_t n, uint64_t first_event,
    struct oracle_state * states, struct oracle_result * results,
    int period, int max_frames, struct oracle_frame * frames, int * length)
{
        if (ref_physics == NULL) return PUMAS_RETURN_PHYSICS_ERROR;
        pumas_error_handler_set(NULL);
        struct ref_medium * media =
            calloc(geometry->n_media > 0 ? geometry->n_media : 1,
                sizeof(*media));
        if (media == NULL) return PUMAS_RETURN_MEMORY_ERROR;
        int i;
        for (i = 0; i < geometry->n_media; i++) {
                media[i].api.material = geometry->media[i].material;
                media[i].density = geometry->media[i].density;
                media[i].loc = (geometry->locals != NULL) ?
                    geometry->locals + i : NULL;
                media[i].api.locals =
                    ((media[i].density > 0.) || (media[i].loc != NULL)) ?
                    &ref_locals : NULL;
        }
        struct pumas_context * context = NULL;
        struct pumas_recorder * recorder = NULL;
        enum pumas_return rc = pumas_context_create(
            &context, ref_physics, sizeof(struct ref_event));
        if (rc == PUMAS_RETURN_SUCCESS)
                rc = pumas_recorder_create(&recorder, 0);
        if (rc != PUMAS_RETURN_SUCCESS) {
                if (context != NULL) pumas_context_destroy(&context);
                free(media);
                return rc;
        }
        recorder->period = period;
        context->recorder = recorder;
        context->medium = &ref_medium_cb;
        context->random = &ref_random;
        context->mode.energy_loss = cfg->energy_loss;
        context->mode.decay = cfg->decay;
        context->mode.direction = cfg->direction;
        context->mode.scattering = cfg->scattering;
        context->event = cfg->event;
        context->limit.energy = cfg->limit_energy;
        context->limit.distance = cfg->limit_distance;
        context->limit.grammage = cfg->limit_grammage;
        context->limit.time = cfg->limit_time;
        context->accuracy = cfg->accuracy;
        struct ref_event * data = context->user_data;
        data->geometry = geometry;
        data->media = media;
        struct simulation_context * context_ =
            (struct simulation_context *)context;
        int64_t k;
        for (k = 0; k < n; k++) {
                data->stream.seed = cfg->seed;
                data->stream.event = first_event + k;
                data->stream.n = 0;
                data->stream.next = 0.;
                data->steps = 0;
                context_->randn_done = 0;
                context_->randn_next = 0.;
                pumas_recorder_clear(recorder);
                enum pumas_event event = PUMAS_EVENT_NONE;
                struct pumas_medium * m[2] = { NULL, NULL };
                const enum pumas_return rck = pumas_context_transport(
                    context, (struct pumas_state *)(states + k), &event, m);
                struct oracle_result * r = results + k;
                r->event = event;
                r->medium_in = (m[0] == NULL) ? -1 :
                    (int)((struct ref_medium *)m[0] - media);
                r->medium_out = (m[1] == NULL) ? -1 :
                    (int)((struct ref_medium *)m[1] - media);
                r->status = rck;
                r->steps = data->steps;
                r->randn_done = context_->randn_done;
                r->draws = data->stream.n;
                r->randn_next = context_->randn_next;
                length[k] = recorder->length;
                const struct pumas_frame * f = recorder->first;
                int j;
                for (j = 0; (j < max_frames) && (f != NULL);
                     j++, f = f->next) {
                        struct oracle_frame * o =
                            frames + k * (int64_t)max_frames + j;
                        memcpy(&o->state, &f->state, sizeof(o->state));
                        o->medium = (f->medium == NULL) ? -1 :
                            (int)((struct ref_medium *)f->medium - media);
                        o->event = f->event;
                }
        }
        pumas_recorder_destroy(&recorder);
        pumas_context_destroy(&context);
        free(media);
        return PUMAS_RETURN_SUCCESS;
}

/* The per element DEL tables computed by the reference's own functions on
 * the loaded physics (its elements, energy grid and DCS models): the
 * restricted cross sections of compute_cel_and_del (pumas.c:10722-10737)
 * and the DCS table rows of compute_dcs_table without the envelope maxima
 * (pumas.c:11629-11699: dcs_tabulate_row and the low energy exponents), in
 * the dump's layouts (see oracle_port_dcs_tables). The DCS table rows read
 * the cross sections of the loaded physics, as in the reference. The wall
 * time of each part goes to seconds[2]. */
int oracle_ref_dcs_tables(double * csn, float * dcs, float * alpha,
    double * seconds)
{
        if (ref_physics == NULL) return PUMAS_RETURN_PHYSICS_ERROR;
        struct pumas_physics * physics = ref_physics;
        const int nel = physics->n_elements, nE = physics->n_energies;
        const int n = physics->n_table_dcs;
        double t0 = omp_get_wtime();
        int ip, iel, row;
        for (ip = 0; ip < N_DEL_PROCESSES; ip++) {
                dcs_function_t * f = dcs_get(ip);
                for (iel = 0; iel < nel; iel++) {
                        for (row = 0; row < nE; row++) {
                                csn[(ip * nel + iel) * nE + row] = (row == 0) ?
                                    0. :
                                    compute_dcs_integral(physics, 0,
                                        physics->element[iel],
                                        physics->table_K[row], f,
                                        physics->cutoff, 1, 180);
                        }
                }
        }
        double t1 = omp_get_wtime();
        seconds[0] = t1 - t0;

        /* The sampling grid and work space of compute_dcs_table. */
        struct dcs_tabulate_work * work =
            malloc(sizeof(*work) + 3 * n * sizeof(*work->x));
        if (work == NULL) return PUMAS_RETURN_MEMORY_ERROR;
        work->x = work->data;
        work->y = work->x + n;
        work->m = work->y + n;
        const int p = DCS_MODEL_N_REVERSE;
        const int m = n - p;
        double xrev;
        int i;
        if (m > 0) {
                xrev = DCS_MODEL_X_REVERSE;
                const double x0 = log(physics->cutoff);
                const double dx = log(xrev / physics->cutoff) / (m - 1);
                for (i = 0; i < m; i++) work->x[i] = x0 + i * dx;
        } else {
                xrev = physics->cutoff;
        }
        const double dxmin = DCS_MODEL_DXMIN;
        const double dx = log((DCS_MODEL_MAX_FRACTION - xrev) / dxmin) /
            ((m > 0) ? p : p - 1);
        for (i = 0; i < p; i++)
                work->x[n - 1 - i] =
                    log(DCS_MODEL_MAX_FRACTION - dxmin * exp(i * dx));
        for (ip = 0; ip < N_DEL_PROCESSES - 1; ip++) {
                for (iel = 0; iel < nel; iel++) {
                        /* Envelopes start at zero, as in a fresh
                         * pumas_physics_create: rows without cross section
                         * are not written by dcs_tabulate_row. */
                        for (row = 0; row < nE; row++)
                                table_get_dcs_envelope(
                                    physics, ip, iel, row)[0] = 0.f;
                        for (row = 0; row < nE; row++)
                                dcs_tabulate_row(physics, ip, iel, row, work);
                        int n0 = 0;
                        float a0 = 0.f;
                        for (row = 0; row < nE; row++) {
                                const float * env = table_get_dcs_envelope(
                                    physics, ip, iel, row);
                                if (env[0] > 0.f) {
                                        n0 = row;
                                        a0 = env[0];
                                        break;
                                }
                        }
                        for (row = 0; row < nE; row++) {
                                const float * env = table_get_dcs_envelope(
                                    physics, ip, iel, row);
                                alpha[(ip * nel + iel) * nE + row] =
                                    (row < n0) ? a0 : env[0];
                        }
                }
        }
        free(work);
        memcpy(dcs, physics->table_DCS,
            (size_t)3 * nel * nE * 2 * n * sizeof(float));
        seconds[1] = omp_get_wtime() - t1;
        return PUMAS_RETURN_SUCCESS;
}

/* The reference's loaded physics itself (a live struct pumas_physics, with
 * pointers into this process) and its size in bytes. */
const void * oracle_ref_physics(int * size)
{
        if (ref_physics == NULL) return NULL;
        memcpy(size, ref_physics, sizeof(*size));
        return ref_physics;
}
