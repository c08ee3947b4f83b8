/*
 * gp_context.h -- host side state of a transport context.
 */
#ifndef GP_CONTEXT_H
#define GP_CONTEXT_H

#include <cuda_runtime.h>

#include "gpumas.h"
#include "gp_internal.h"

struct gpumas_engine;

/* Engine parameters (gpumas_tuning of gpumas.h). */
struct gp_tuning {
        int engine;      /* 0: automatic, 1: one thread per event, 2: pool */
        int pool_slots;  /* number of event slots of the pool engine */
        int max_inner;   /* continuous steps per slot and iteration */
        int batch;       /* iterations per captured graph */
        int tail;        /* drain threshold in slots (0: off, <0: automatic) */
};

struct gp_context {
        struct gpumas_context api; /* first member: public view */
        const struct gpumas_physics * physics;
        gp_tables * d_tables;
        gpumas_geometry * d_geometry;
        void * d_geometry_data;
        int has_geometry;
        int n_media;
        int geometry_kind;
        int has_locals; /* media with local properties: ext kernel only */
        void * d_io;
        size_t io_size;
        cudaStream_t stream;
        cudaEvent_t t0, t1;
        struct gpumas_stats stats;
        void * extra;
        struct gpumas_engine * pool; /* slot pool engine of the context */
        struct gp_tuning tuning;
        struct gpumas_recorder recorder; /* frames, if recording */
        int recording;
        int max_trials; /* rejection sampling cap (gp_config.max_trials) */
        int carry;      /* continue events across calls (gp_config.carry) */
};


static inline int gp_check(cudaError_t rc)
{
        return (rc == cudaSuccess) ? GPUMAS_RETURN_SUCCESS :
                                     GPUMAS_RETURN_DEVICE_ERROR;
}

#ifdef __cplusplus
extern "C" {
#endif
void gp_pool_free(struct gpumas_engine * engine);
#ifdef __cplusplus
}
#endif

#endif
