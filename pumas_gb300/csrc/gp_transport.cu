/*
 * gp_transport.cu -- transport kernels and the context C ABI.
 *
 * Replaces the per event `pumas_context_transport` loop of a user program
 * (e.g. the reference's examples/pumas/straight.c:133-179) by batched
 * launches: one GPU thread per event, the event state in registers, the
 * physics image and the geometry descriptor read through the L1 / L2
 * caches. Context level checks mirror pumas.c:3120-3177 and are done on the
 * host before any launch; per event checks (direction norm, density) are
 * done on the device and reported in the per event status.
 */
#include <cuda_runtime.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "gp_device.cuh"

#include "gp_io.cuh"
#include "gp_context.h"

extern "C" int gp_pool_transport(gp_context * c, const gp_config * cfg,
    const gp_io * io, size_t n, uint64_t first, cudaStream_t s,
    const gp_tuning * tuning, int * launches);

/* One thread per event, the whole transport call in one launch. */
__global__ void __launch_bounds__(128, 1) gp_kernel_plain(
    const gp_tables * __restrict__ Tp, const gp_config cfg,
    const gpumas_geometry * __restrict__ gp, const gp_io io, size_t n,
    uint64_t first_event)
{
        const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
        if (i >= n) return;
        const gp_tables & T = *Tp;
        const gpumas_geometry & g = *gp;
        gp_event e;
        io.begin(i, cfg, first_event + i, e);
        int event, m_in, m_out;
        gp_transport(T, cfg, g, e, event, m_in, m_out);
        io.store(i, e, event, m_in, m_out);
}

/* One thread per event with the frame recorder (struct pumas_recorder,
 * pumas.h:432-458) and / or the media's local properties (density profiles
 * and magnetic fields, struct gpumas_locals). With the recorder, event i
 * writes its frames after those of events 0 .. i - 1, max_frames each. */
__global__ void __launch_bounds__(128, 1) gp_kernel_plain_ext(
    const gp_tables * __restrict__ Tp, const gp_config cfg,
    const gpumas_geometry * __restrict__ gp, const gp_io io, size_t n,
    uint64_t first_event, const gpumas_recorder recorder, int recording,
    int locals)
{
        const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
        if (i >= n) return;
        const gp_tables & T = *Tp;
        const gpumas_geometry & g = *gp;
        gp_event e;
        io.begin(i, cfg, first_event + i, e);
        gp_rec r;
        r.frames = recording ?
            recorder.frames + i * (size_t)recorder.max_frames : NULL;
        r.max_frames = recorder.max_frames;
        r.period = recorder.period;
        r.count = 0;
        gp_loc l;
        int event, m_in, m_out;
        gp_transport(T, cfg, g, e, event, m_in, m_out,
            recording ? &r : NULL, locals ? &l : NULL);
        io.store(i, e, event, m_in, m_out);
        if (recording) recorder.length[i] = r.count;
}

/* Draws of the Philox stream, for checking against other implementations. */
__global__ void gp_kernel_random(uint64_t seed, uint32_t domain,
    uint64_t event, uint64_t first, size_t n, double * out)
{
        const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
        if (i >= n) return;
        const uint64_t k = first + i;
        uint32_t x[4];
        gp_philox((uint32_t)(k >> 1), domain, (uint32_t)event,
            (uint32_t)(event >> 32), (uint32_t)seed, (uint32_t)(seed >> 32),
            x);
        out[i] = (k & 1) ? gp_word_to_uniform(x[2], x[3]) :
                           gp_word_to_uniform(x[0], x[1]);
}

/* ------------------------------------------------------------------------ */
/* Contexts.                                                                */
/* ------------------------------------------------------------------------ */

extern "C" int gp_api_context_create(struct gpumas_context ** context,
    const struct gpumas_physics * physics, int extra_memory)
{
        if (context == NULL) return GPUMAS_RETURN_VALUE_ERROR;
        *context = NULL;
        if (physics == NULL) return GPUMAS_RETURN_PHYSICS_ERROR;
        gp_context * c = (gp_context *)calloc(1, sizeof(*c));
        if (c == NULL) return GPUMAS_RETURN_MEMORY_ERROR;
        c->physics = physics;
        /* Defaults of pumas_context_create (pumas.c:2592-2612). */
        c->api.mode.energy_loss = GPUMAS_MODE_STRAGGLED;
        c->api.mode.decay = (physics->particle == GPUMAS_PARTICLE_MUON) ?
            GPUMAS_MODE_WEIGHTED : GPUMAS_MODE_RANDOMISED;
        c->api.mode.direction = GPUMAS_MODE_FORWARD;
        c->api.mode.scattering = GPUMAS_MODE_MIXED;
        c->api.event = GPUMAS_EVENT_NONE;
        c->api.accuracy = 1E-02;
        c->api.seed = 0;
        c->tuning.engine = 0;
        c->tuning.pool_slots = 1048576;
        c->tuning.max_inner = 8;
        c->tuning.batch = 16;
        c->tuning.tail = 0;
        c->max_trials = GP_MAX_REJECTIONS_DEFAULT;
        if (extra_memory > 0) {
                c->extra = calloc(1, extra_memory);
                c->api.user_data = c->extra;
        }
        gp_tables tables;
        gp_physics_tables(physics, &tables);
        int rc = gp_check(cudaMalloc(&c->d_tables, sizeof(gp_tables)));
        if (rc == GPUMAS_RETURN_SUCCESS)
                rc = gp_check(cudaMemcpy(c->d_tables, &tables,
                    sizeof(gp_tables), cudaMemcpyHostToDevice));
        if (rc == GPUMAS_RETURN_SUCCESS)
                rc = gp_check(cudaMalloc(&c->d_geometry,
                    sizeof(gpumas_geometry)));
        if (rc == GPUMAS_RETURN_SUCCESS)
                rc = gp_check(cudaStreamCreateWithFlags(
                    &c->stream, cudaStreamNonBlocking));
        if (rc == GPUMAS_RETURN_SUCCESS)
                rc = gp_check(cudaEventCreate(&c->t0));
        if (rc == GPUMAS_RETURN_SUCCESS)
                rc = gp_check(cudaEventCreate(&c->t1));
        if (rc != GPUMAS_RETURN_SUCCESS) {
                struct gpumas_context * tmp = &c->api;
                gpumas_context_destroy(&tmp);
                return rc;
        }
        *context = &c->api;
        return GPUMAS_RETURN_SUCCESS;
}

extern "C" int gp_api_context_random_seed_set(
    struct gpumas_context * context, const uint64_t * seed)
{
        if (context == NULL) return GPUMAS_RETURN_VALUE_ERROR;
        if (seed != NULL) {
                context->seed = *seed;
                return GPUMAS_RETURN_SUCCESS;
        }
        FILE * stream = fopen("/dev/urandom", "rb");
        if (stream == NULL) return GPUMAS_RETURN_PATH_ERROR;
        uint64_t s;
        const size_t n = fread(&s, sizeof(s), 1, stream);
        fclose(stream);
        if (n != 1) return GPUMAS_RETURN_PATH_ERROR;
        context->seed = s;
        return GPUMAS_RETURN_SUCCESS;
}

extern "C" int gp_api_context_random_seed_get(
    const struct gpumas_context * context, uint64_t * seed)
{
        if ((context == NULL) || (seed == NULL))
                return GPUMAS_RETURN_VALUE_ERROR;
        *seed = context->seed;
        return GPUMAS_RETURN_SUCCESS;
}

extern "C" const struct gpumas_physics * gpumas_context_physics_get(
    const struct gpumas_context * context)
{
        if (context == NULL) return NULL;
        return ((const gp_context *)context)->physics;
}

extern "C" void gpumas_context_destroy(struct gpumas_context ** context)
{
        if ((context == NULL) || (*context == NULL)) return;
        gp_context * c = (gp_context *)(*context);
        if (c->d_tables != NULL) cudaFree(c->d_tables);
        if (c->d_geometry != NULL) cudaFree(c->d_geometry);
        if (c->d_geometry_data != NULL) cudaFree(c->d_geometry_data);
        if (c->d_io != NULL) cudaFree(c->d_io);
        gp_pool_free(c->pool);
        if (c->stream != NULL) cudaStreamDestroy(c->stream);
        if (c->t0 != NULL) cudaEventDestroy(c->t0);
        if (c->t1 != NULL) cudaEventDestroy(c->t1);
        free(c->extra);
        free(c);
        *context = NULL;
}

/* Copy a geometry descriptor and its arrays to one device allocation. */
extern "C" int gp_geometry_upload(const struct gpumas_physics * physics,
    const struct gpumas_geometry * geometry, gpumas_geometry * d_geometry,
    void ** d_data)
{
        if (geometry == NULL) return GPUMAS_RETURN_MEDIUM_ERROR;
        const gpumas_geometry & g = *geometry;
        if ((g.n_media <= 0) || (g.media == NULL))
                return GPUMAS_RETURN_MEDIUM_ERROR;
        for (int i = 0; i < g.n_media; i++) {
                if ((g.media[i].material < 0) ||
                    (g.media[i].material >= physics->n_materials))
                        return GPUMAS_RETURN_INDEX_ERROR;
        }
        size_t sz_media = g.n_media * sizeof(gpumas_medium);
        size_t sz_z = 0, sz_m = 0, sz_h = 0, sz_l = 0;
        if (g.locals != NULL) {
                for (int i = 0; i < g.n_media; i++) {
                        const gpumas_locals & l = g.locals[i];
                        for (int k = 0; k < 3; k++)
                                if (!isfinite(l.magnet[k]))
                                        return GPUMAS_RETURN_VALUE_ERROR;
                        if (l.model == GPUMAS_DENSITY_UNIFORM) continue;
                        if (l.model != GPUMAS_DENSITY_EXPONENTIAL)
                                return GPUMAS_RETURN_VALUE_ERROR;
                        if (!(l.rho0 > 0.) || !(l.lambda > 0.) ||
                            !(l.eps > 0.) || !isfinite(l.h0) ||
                            !isfinite(l.rho0) || !isfinite(l.lambda))
                                return GPUMAS_RETURN_VALUE_ERROR;
                        for (int k = 0; k < 3; k++)
                                if (!isfinite(l.axis[k]))
                                        return GPUMAS_RETURN_VALUE_ERROR;
                }
                sz_l = g.n_media * sizeof(gpumas_locals);
        }
        if (g.kind == GPUMAS_GEOMETRY_UNIFORM) {
                if ((g.uniform_medium < 0) || (g.uniform_medium >= g.n_media))
                        return GPUMAS_RETURN_INDEX_ERROR;
        } else if (g.kind == GPUMAS_GEOMETRY_SLABS) {
                if ((g.n_slabs <= 0) || (g.slab_z == NULL) ||
                    (g.slab_medium == NULL))
                        return GPUMAS_RETURN_MEDIUM_ERROR;
                for (int i = 0; i < g.n_slabs; i++) {
                        if (!(g.slab_z[i] < g.slab_z[i + 1]))
                                return GPUMAS_RETURN_VALUE_ERROR;
                        if ((g.slab_medium[i] < -1) ||
                            (g.slab_medium[i] >= g.n_media))
                                return GPUMAS_RETURN_INDEX_ERROR;
                }
                sz_z = (g.n_slabs + 1) * sizeof(double);
                sz_m = g.n_slabs * sizeof(int);
        } else if (g.kind == GPUMAS_GEOMETRY_HEIGHTMAP) {
                if ((g.hm_nx < 2) || (g.hm_ny < 2) || (g.hm_z == NULL) ||
                    !(g.hm_dx > 0.) || !(g.hm_dy > 0.))
                        return GPUMAS_RETURN_VALUE_ERROR;
                if ((g.hm_below < -1) || (g.hm_below >= g.n_media) ||
                    (g.hm_above < -1) || (g.hm_above >= g.n_media))
                        return GPUMAS_RETURN_INDEX_ERROR;
                sz_h = (size_t)g.hm_nx * g.hm_ny * sizeof(double);
        } else {
                return GPUMAS_RETURN_VALUE_ERROR;
        }
        const size_t o_media = 0;
        const size_t o_z = (o_media + sz_media + 255) & ~(size_t)255;
        const size_t o_m = (o_z + sz_z + 255) & ~(size_t)255;
        const size_t o_h = (o_m + sz_m + 255) & ~(size_t)255;
        const size_t o_l = (o_h + sz_h + 255) & ~(size_t)255;
        const size_t total = o_l + sz_l;
        char * host = (char *)calloc(1, total);
        if (host == NULL) return GPUMAS_RETURN_MEMORY_ERROR;
        memcpy(host + o_media, g.media, sz_media);
        if (sz_z) memcpy(host + o_z, g.slab_z, sz_z);
        if (sz_m) memcpy(host + o_m, g.slab_medium, sz_m);
        if (sz_h) memcpy(host + o_h, g.hm_z, sz_h);
        if (sz_l) memcpy(host + o_l, g.locals, sz_l);
        char * d = NULL;
        int rc = gp_check(cudaMalloc(&d, total));
        if (rc == GPUMAS_RETURN_SUCCESS)
                rc = gp_check(
                    cudaMemcpy(d, host, total, cudaMemcpyHostToDevice));
        free(host);
        if (rc != GPUMAS_RETURN_SUCCESS) {
                if (d != NULL) cudaFree(d);
                return rc;
        }
        gpumas_geometry dg = g;
        dg.media = (const gpumas_medium *)(d + o_media);
        dg.slab_z = sz_z ? (const double *)(d + o_z) : NULL;
        dg.slab_medium = sz_m ? (const int *)(d + o_m) : NULL;
        dg.hm_z = sz_h ? (const double *)(d + o_h) : NULL;
        dg.locals = sz_l ? (const gpumas_locals *)(d + o_l) : NULL;
        rc = gp_check(cudaMemcpy(
            d_geometry, &dg, sizeof(dg), cudaMemcpyHostToDevice));
        if (rc != GPUMAS_RETURN_SUCCESS) {
                cudaFree(d);
                return rc;
        }
        *d_data = d;
        return GPUMAS_RETURN_SUCCESS;
}

extern "C" int gp_api_context_geometry_set(
    struct gpumas_context * context, const struct gpumas_geometry * geometry)
{
        if (context == NULL) return GPUMAS_RETURN_VALUE_ERROR;
        gp_context * c = (gp_context *)context;
        void * data = NULL;
        const int rc =
            gp_geometry_upload(c->physics, geometry, c->d_geometry, &data);
        if (rc != GPUMAS_RETURN_SUCCESS) return rc;
        if (c->d_geometry_data != NULL) cudaFree(c->d_geometry_data);
        c->d_geometry_data = data;
        c->has_geometry = 1;
        c->n_media = geometry->n_media;
        c->geometry_kind = geometry->kind;
        c->has_locals = (geometry->locals != NULL);
        return GPUMAS_RETURN_SUCCESS;
}

/* Context level checks of pumas_context_transport (pumas.c:3120-3177). */
extern "C" int gp_config_check(const struct gpumas_context * context,
    const struct gpumas_physics * physics, gp_config * cfg)
{
        if (context->mode.direction != GPUMAS_MODE_FORWARD &&
            context->mode.direction != GPUMAS_MODE_BACKWARD)
                return GPUMAS_RETURN_VALUE_ERROR;
        if ((context->mode.energy_loss < GPUMAS_MODE_DISABLED) ||
            (context->mode.energy_loss > GPUMAS_MODE_STRAGGLED))
                return GPUMAS_RETURN_VALUE_ERROR;
        if ((context->mode.scattering != GPUMAS_MODE_DISABLED) &&
            (context->mode.scattering != GPUMAS_MODE_MIXED))
                return GPUMAS_RETURN_VALUE_ERROR;
        if ((context->mode.decay < GPUMAS_MODE_DISABLED) ||
            (context->mode.decay > GPUMAS_MODE_RANDOMISED))
                return GPUMAS_RETURN_DECAY_ERROR;
        /* Weighted decay is invalid for forward taus (pumas.c:3157-3161). */
        if ((physics->particle == GPUMAS_PARTICLE_TAU) &&
            (context->mode.direction == GPUMAS_MODE_FORWARD) &&
            (context->mode.decay == GPUMAS_MODE_WEIGHTED))
                return GPUMAS_RETURN_DECAY_ERROR;
        if ((context->accuracy <= 0) || (context->accuracy > 1))
                return GPUMAS_RETURN_ACCURACY_ERROR;
        if ((context->mode.direction == GPUMAS_MODE_BACKWARD) &&
            (context->mode.energy_loss > GPUMAS_MODE_CSDA) &&
            (physics->tables.cutoff < 1E-02))
                return GPUMAS_RETURN_ACCURACY_ERROR;
        cfg->energy_loss = context->mode.energy_loss;
        cfg->decay = context->mode.decay;
        cfg->direction = context->mode.direction;
        cfg->scattering = context->mode.scattering;
        cfg->event = context->event;
        cfg->limit_energy = context->limit.energy;
        cfg->limit_distance = context->limit.distance;
        cfg->limit_grammage = context->limit.grammage;
        cfg->limit_time = context->limit.time;
        cfg->accuracy = context->accuracy;
        cfg->seed = context->seed;
        cfg->max_trials = ((const gp_context *)context)->max_trials;
        cfg->carry = ((const gp_context *)context)->carry;
        return GPUMAS_RETURN_SUCCESS;
}

static const int gp_block = 128;

/* Whether events of this configuration can ever take a step: CSDA without
 * scattering in a uniform infinite medium is the closed form of
 * transport_with_csda (pumas.c:3220-3246). */
static int gp_needs_stepping(const gp_context * c, const gp_config & cfg)
{
        return !((c->geometry_kind == GPUMAS_GEOMETRY_UNIFORM) &&
            (cfg.energy_loss == GPUMAS_MODE_CSDA) &&
            (cfg.scattering == GPUMAS_MODE_DISABLED));
}

/* Run a transport of n events of `io` on stream s with the context's
 * engine. */
static int gp_run(gp_context * c, const gp_config & cfg, const gp_io & io,
    size_t n, uint64_t first_event, cudaStream_t s, int sync)
{
        int engine = c->tuning.engine;
        if (engine == 0) engine = gp_needs_stepping(c, cfg) ? 2 : 1;
        int rc;
        cudaEventRecord(c->t0, s);
        /* The recorder runs on the one thread per event kernel; media with
         * local properties run on it or on the slot pool. */
        if (c->recording || (c->has_locals && (engine != 2))) {
                const unsigned int grid =
                    (unsigned int)((n + gp_block - 1) / gp_block);
                gp_kernel_plain_ext<<<grid, gp_block, 0, s>>>(c->d_tables,
                    cfg, c->d_geometry, io, n, first_event, c->recorder,
                    c->recording, c->has_locals);
                rc = gp_check(cudaGetLastError());
                c->stats.launches = 1;
        } else if (engine == 2) {
                int launches = 0;
                rc = gp_pool_transport(
                    c, &cfg, &io, n, first_event, s, &c->tuning, &launches);
                c->stats.launches = launches;
        } else {
                const unsigned int grid =
                    (unsigned int)((n + gp_block - 1) / gp_block);
                gp_kernel_plain<<<grid, gp_block, 0, s>>>(
                    c->d_tables, cfg, c->d_geometry, io, n, first_event);
                rc = gp_check(cudaGetLastError());
                c->stats.launches = 1;
        }
        cudaEventRecord(c->t1, s);
        c->stats.kernel_ms = -1.;
        if ((rc == 0) && sync) rc = gp_check(cudaStreamSynchronize(s));
        return rc;
}

extern "C" int gp_api_context_recorder_set(
    struct gpumas_context * context, const struct gpumas_recorder * recorder)
{
        if (context == NULL) return GPUMAS_RETURN_VALUE_ERROR;
        gp_context * c = (gp_context *)context;
        if (recorder == NULL) {
                c->recording = 0;
                memset(&c->recorder, 0, sizeof(c->recorder));
                return GPUMAS_RETURN_SUCCESS;
        }
        if ((recorder->max_frames < 0) || (recorder->length == NULL) ||
            ((recorder->max_frames > 0) && (recorder->frames == NULL)))
                return GPUMAS_RETURN_VALUE_ERROR;
        c->recorder = *recorder;
        c->recording = 1;
        return GPUMAS_RETURN_SUCCESS;
}

extern "C" int gp_api_context_tuning_set(
    struct gpumas_context * context, const struct gpumas_tuning * tuning)
{
        if ((context == NULL) || (tuning == NULL))
                return GPUMAS_RETURN_VALUE_ERROR;
        gp_context * c = (gp_context *)context;
        if ((tuning->engine < 0) || (tuning->engine > 2) ||
            (tuning->pool_slots < 0) || (tuning->max_inner < 0) ||
            (tuning->batch < 0))
                return GPUMAS_RETURN_VALUE_ERROR;
        if (tuning->engine != 0) c->tuning.engine = tuning->engine;
        if (tuning->pool_slots > 0) c->tuning.pool_slots = tuning->pool_slots;
        if (tuning->max_inner > 0) c->tuning.max_inner = tuning->max_inner;
        if (tuning->batch > 0) c->tuning.batch = tuning->batch;
        if (tuning->tail != 0) c->tuning.tail = tuning->tail;
        return GPUMAS_RETURN_SUCCESS;
}

extern "C" int gp_api_context_trials_set(
    struct gpumas_context * context, int max_trials)
{
        if ((context == NULL) || (max_trials < 0))
                return GPUMAS_RETURN_VALUE_ERROR;
        ((gp_context *)context)->max_trials = (max_trials > 0) ?
            max_trials : GP_MAX_REJECTIONS_DEFAULT;
        return GPUMAS_RETURN_SUCCESS;
}

extern "C" int gp_api_context_carry_set(
    struct gpumas_context * context, int carry)
{
        if ((context == NULL) || (carry < 0) || (carry > 1))
                return GPUMAS_RETURN_VALUE_ERROR;
        ((gp_context *)context)->carry = carry;
        return GPUMAS_RETURN_SUCCESS;
}

extern "C" int gp_api_context_carry_get(
    const struct gpumas_context * context, int * carry)
{
        if ((context == NULL) || (carry == NULL))
                return GPUMAS_RETURN_VALUE_ERROR;
        *carry = ((const gp_context *)context)->carry;
        return GPUMAS_RETURN_SUCCESS;
}

extern "C" int gp_api_context_trials_get(
    const struct gpumas_context * context, int * max_trials)
{
        if ((context == NULL) || (max_trials == NULL))
                return GPUMAS_RETURN_VALUE_ERROR;
        *max_trials = ((const gp_context *)context)->max_trials;
        return GPUMAS_RETURN_SUCCESS;
}

extern "C" int gp_api_context_tuning_get(
    const struct gpumas_context * context, struct gpumas_tuning * tuning)
{
        if ((context == NULL) || (tuning == NULL))
                return GPUMAS_RETURN_VALUE_ERROR;
        const gp_context * c = (const gp_context *)context;
        tuning->engine = c->tuning.engine;
        tuning->pool_slots = c->tuning.pool_slots;
        tuning->max_inner = c->tuning.max_inner;
        tuning->batch = c->tuning.batch;
        tuning->tail = c->tuning.tail;
        return GPUMAS_RETURN_SUCCESS;
}

extern "C" int gp_api_context_transport_device(struct gpumas_context * context,
    size_t n, const struct gpumas_soa * events, uint64_t first_event,
    void * stream)
{
        if ((context == NULL) || (events == NULL))
                return GPUMAS_RETURN_VALUE_ERROR;
        gp_context * c = (gp_context *)context;
        if (!c->has_geometry) return GPUMAS_RETURN_MEDIUM_ERROR;
        gp_config cfg;
        int rc = gp_config_check(context, c->physics, &cfg);
        if (rc != GPUMAS_RETURN_SUCCESS) return rc;
        if (n == 0) return GPUMAS_RETURN_SUCCESS;
        if (cfg.carry && (events->result == NULL))
                return GPUMAS_RETURN_VALUE_ERROR;
        gp_io io;
        memset(&io, 0, sizeof(io));
        io.soa.a = *events;
        return gp_run(c, cfg, io, n, first_event, (cudaStream_t)stream, 0);
}

extern "C" int gp_api_context_transport(struct gpumas_context * context,
    size_t n, struct gpumas_state * states, struct gpumas_result * results,
    uint64_t first_event)
{
        if (context == NULL) return GPUMAS_RETURN_VALUE_ERROR;
        gp_context * c = (gp_context *)context;
        if (!c->has_geometry) return GPUMAS_RETURN_MEDIUM_ERROR;
        gp_config cfg;
        int rc = gp_config_check(context, c->physics, &cfg);
        if (rc != GPUMAS_RETURN_SUCCESS) return rc;
        if (n == 0) return GPUMAS_RETURN_SUCCESS;
        if (states == NULL) return GPUMAS_RETURN_VALUE_ERROR;
        if (cfg.carry && (results == NULL)) return GPUMAS_RETURN_VALUE_ERROR;

        const size_t sz_s = n * sizeof(gpumas_state);
        const size_t sz_r = n * sizeof(gpumas_result);
        const size_t o_r = (sz_s + 255) & ~(size_t)255;
        const size_t need = o_r + sz_r;
        if (need > c->io_size) {
                if (c->d_io != NULL) cudaFree(c->d_io);
                c->d_io = NULL;
                c->io_size = 0;
                rc = gp_check(cudaMalloc(&c->d_io, need));
                if (rc != GPUMAS_RETURN_SUCCESS) return rc;
                c->io_size = need;
        }
        gp_io io;
        memset(&io, 0, sizeof(io));
        io.aos.states = (gpumas_state *)c->d_io;
        io.aos.results = (gpumas_result *)((char *)c->d_io + o_r);
        cudaStream_t s = c->stream;
        rc = gp_check(cudaMemcpyAsync(
            io.aos.states, states, sz_s, cudaMemcpyHostToDevice, s));
        if ((rc == GPUMAS_RETURN_SUCCESS) && cfg.carry)
                rc = gp_check(cudaMemcpyAsync(io.aos.results, results, sz_r,
                    cudaMemcpyHostToDevice, s));
        if (rc != GPUMAS_RETURN_SUCCESS) return rc;
        rc = gp_run(c, cfg, io, n, first_event, s, 0);
        if (rc != GPUMAS_RETURN_SUCCESS) return rc;
        rc = gp_check(cudaMemcpyAsync(
            states, io.aos.states, sz_s, cudaMemcpyDeviceToHost, s));
        if (rc != GPUMAS_RETURN_SUCCESS) return rc;
        gpumas_result * hr = results;
        gpumas_result * tmp = NULL;
        if (hr == NULL) {
                tmp = (gpumas_result *)malloc(sz_r);
                if (tmp == NULL) return GPUMAS_RETURN_MEMORY_ERROR;
                hr = tmp;
        }
        rc = gp_check(cudaMemcpyAsync(
            hr, io.aos.results, sz_r, cudaMemcpyDeviceToHost, s));
        if (rc == GPUMAS_RETURN_SUCCESS)
                rc = gp_check(cudaStreamSynchronize(s));
        float ms = 0.f;
        cudaEventElapsedTime(&ms, c->t0, c->t1);
        c->stats.kernel_ms = ms;
        if (rc == GPUMAS_RETURN_SUCCESS) {
                for (size_t i = 0; i < n; i++) {
                        if (hr[i].status != GPUMAS_RETURN_SUCCESS) {
                                rc = hr[i].status;
                                break;
                        }
                }
        }
        free(tmp);
        return rc;
}

extern "C" int gp_api_context_stats(
    const struct gpumas_context * context, struct gpumas_stats * stats)
{
        if ((context == NULL) || (stats == NULL))
                return GPUMAS_RETURN_VALUE_ERROR;
        const gp_context * c = (const gp_context *)context;
        *stats = c->stats;
        if (stats->kernel_ms < 0.) {
                float ms = 0.f;
                if (cudaEventElapsedTime(&ms, c->t0, c->t1) == cudaSuccess)
                        stats->kernel_ms = ms;
        }
        return GPUMAS_RETURN_SUCCESS;
}

/* FP64 throughput microbenchmark: 8 independent DFMA chains per thread. */
__global__ void gp_kernel_dfma(double * out, int iters, double a, double b)
{
        double x[8];
#pragma unroll
        for (int k = 0; k < 8; k++) x[k] = threadIdx.x * 1E-03 + k;
        for (int i = 0; i < iters; i++) {
#pragma unroll
                for (int k = 0; k < 8; k++) x[k] = fma(x[k], a, b);
        }
        double s = 0.;
#pragma unroll
        for (int k = 0; k < 8; k++) s += x[k];
        if (s == 12345.678) out[0] = s;
}

extern "C" int gp_api_bench_dfma(double * tflops)
{
        if (tflops == NULL) return GPUMAS_RETURN_VALUE_ERROR;
        int device, sms = 0;
        cudaGetDevice(&device);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
        double * d = NULL;
        int rc = gp_check(cudaMalloc(&d, sizeof(double)));
        if (rc != GPUMAS_RETURN_SUCCESS) return rc;
        const int threads = 256, blocks = 8 * sms, iters = 4096;
        cudaEvent_t t0, t1;
        cudaEventCreate(&t0);
        cudaEventCreate(&t1);
        gp_kernel_dfma<<<blocks, threads>>>(d, iters, 0.999999, 1E-07);
        cudaEventRecord(t0);
        gp_kernel_dfma<<<blocks, threads>>>(d, iters, 0.999999, 1E-07);
        cudaEventRecord(t1);
        rc = gp_check(cudaEventSynchronize(t1));
        float ms = 0.f;
        cudaEventElapsedTime(&ms, t0, t1);
        cudaEventDestroy(t0);
        cudaEventDestroy(t1);
        cudaFree(d);
        const double flops = 2. * 8. * iters * (double)threads * blocks;
        *tflops = (ms > 0.f) ? flops / (ms * 1E-03) * 1E-12 : 0.;
        return rc;
}

/* The engine's elementary functions on the device, for checking. */
__global__ void gp_kernel_math(int fn, size_t n, const double * x, double * y)
{
        const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
        if (i >= n) return;
        if (fn == 2) {
                const double * a = x + 4 * i;
                y[i] = gp_neglog_beyond(a[0], a[1], a[2], a[3]);
        } else if (fn >= 3) {
                const float f = (float)x[i];
                y[i] = (fn == 3) ? gp_libm_logf(f) : gp_libm_expf(f);
        } else {
                y[i] = (fn == 0) ? gp_log(x[i]) : gp_exp(x[i]);
        }
}

extern "C" int gp_api_math_eval(int fn, size_t n, const double * x,
    double * y)
{
        if ((x == NULL) || (y == NULL) || (n == 0) || (fn < 0) || (fn > 4))
                return GPUMAS_RETURN_VALUE_ERROR;
        const size_t nx = (fn == 2) ? 4 * n : n;
        double * d = NULL;
        int rc = gp_check(cudaMalloc(&d, (nx + n) * sizeof(double)));
        if (rc != GPUMAS_RETURN_SUCCESS) return rc;
        rc = gp_check(cudaMemcpy(d, x, nx * sizeof(double),
            cudaMemcpyHostToDevice));
        if (rc == GPUMAS_RETURN_SUCCESS) {
                gp_kernel_math<<<(unsigned int)((n + 255) / 256), 256>>>(
                    fn, n, d, d + nx);
                rc = gp_check(cudaGetLastError());
        }
        if (rc == GPUMAS_RETURN_SUCCESS)
                rc = gp_check(cudaMemcpy(y, d + nx, n * sizeof(double),
                    cudaMemcpyDeviceToHost));
        cudaFree(d);
        return rc;
}

extern "C" int gp_api_random_fill(uint64_t seed, uint32_t domain,
    uint64_t event, uint64_t first, size_t n, double * out)
{
        if ((out == NULL) || (n == 0)) return GPUMAS_RETURN_VALUE_ERROR;
        double * d = NULL;
        int rc = gp_check(cudaMalloc(&d, n * sizeof(double)));
        if (rc != GPUMAS_RETURN_SUCCESS) return rc;
        gp_kernel_random<<<(unsigned int)((n + 255) / 256), 256>>>(
            seed, domain, event, first, n, d);
        rc = gp_check(cudaGetLastError());
        if (rc == GPUMAS_RETURN_SUCCESS)
                rc = gp_check(cudaMemcpy(
                    out, d, n * sizeof(double), cudaMemcpyDeviceToHost));
        cudaFree(d);
        return rc;
}
