/*
 * oracle.h -- batch interface of the CPU oracles (test infrastructure only).
 *
 * Two CPU implementations of the `pumas_context_transport` hot path sit
 * behind this interface, with identical signatures:
 *   - oracle_ref_*  : the reference library itself (src/pumas.c compiled
 *                     unmodified from its source tree, see ref_harness.c),
 *                     available where the reference sources are;
 *   - oracle_port_* : a plain C restatement of the same algorithm
 *                     (port.c), which builds anywhere.
 * Both drive one event at a time exactly as a user loop around
 * `pumas_context_transport` (pumas.h:1046-1048) would, with the Philox stream
 * of philox.h as the random callback and the geometries of gpumas_geometry.h
 * as the medium callback. They exist to check the GPU engine, never to run
 * in its place.
 */
#ifndef ORACLE_H
#define ORACLE_H

#include <stdint.h>

#include "gpumas_geometry.h"

/* Same layout as struct pumas_state (pumas.h:289-309). */
struct oracle_state {
        double charge;
        double energy;
        double distance;
        double grammage;
        double time;
        double weight;
        double position[3];
        double direction[3];
        int decayed;
};

/* The public settings of a pumas_context (pumas.h:636-672). */
struct oracle_config {
        int energy_loss;
        int decay;
        int direction;
        int scattering;
        int event;
        double limit_energy;
        double limit_distance;
        double limit_grammage;
        double limit_time;
        double accuracy;
        uint64_t seed;
        /* Each event continues the random stream and Box-Muller cache of
         * its previous call, read from its oracle_result entry, as one
         * reference context per event kept across calls would. */
        int carry;
};

/* Per event outputs besides the state. */
struct oracle_result {
        int event;      /* the transport end event (enum pumas_event) */
        int medium_in;  /* start medium index, -1 for none */
        int medium_out; /* end medium index, -1 for none */
        int status;     /* enum pumas_return of the transport call */
        int steps;      /* number of geometric step proposals */
        int randn_done; /* Box-Muller cache at the end of the call */
        uint64_t draws; /* stream position: random draws since the start */
        double randn_next;
};

/* A recorded frame (struct pumas_frame, pumas.h:378-395) with the medium
 * as an index, -1 for none. Same layout as struct gpumas_frame. */
struct oracle_frame {
        struct oracle_state state;
        int medium;
        int event;
};

#endif
