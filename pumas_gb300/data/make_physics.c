/*
 * make_physics.c -- builds the physics tables consumed by the GPU engine.
 *
 * The GPU engine does not tabulate physics itself: like any user of the
 * reference library it takes the tables produced by the reference's
 * `pumas_physics_create` (pumas.h:898-901) and serialised by
 * `pumas_physics_dump` (pumas.h:929-930). This program is that step. It is
 * compiled against the reference sources by make_physics.sh and writes the
 * dump that is shipped as package data, so that machines without the
 * reference can still load the tables.
 *
 * usage: make_physics <materials.xml> <dedx directory> <output dump>
 *            [muon|tau [<bremsstrahlung> <pair production> <photonuclear>]]
 *
 * The optional model names select the DCS models of
 * struct pumas_physics_settings (pumas.h:721-815); the default is SSR, SSR,
 * DRSS.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "pumas.h"

int main(int argc, char * argv[])
{
        if (argc < 4) {
                fprintf(stderr, "usage: %s <mdf> <dedx dir> <dump>\n", argv[0]);
                return EXIT_FAILURE;
        }
        struct pumas_physics * physics = NULL;
        const enum pumas_particle particle =
            ((argc > 4) && (strcmp(argv[4], "tau") == 0)) ?
            PUMAS_PARTICLE_TAU : PUMAS_PARTICLE_MUON;
        struct pumas_physics_settings settings = { 0 };
        if (argc > 7) {
                settings.bremsstrahlung = argv[5];
                settings.pair_production = argv[6];
                settings.photonuclear = argv[7];
        }
        if (pumas_physics_create(&physics, particle, argv[1], argv[2],
                &settings) != PUMAS_RETURN_SUCCESS)
                return EXIT_FAILURE;
        FILE * stream = fopen(argv[3], "wb");
        if (stream == NULL) return EXIT_FAILURE;
        const int rc = pumas_physics_dump(physics, stream);
        fclose(stream);
        pumas_physics_destroy(&physics);
        return (rc == PUMAS_RETURN_SUCCESS) ? EXIT_SUCCESS : EXIT_FAILURE;
}
