/*
 * sciara_headless_main.cpp -- headless driver for the reference's SCIARA-fv2
 * example (OpenCAL-OMP/examples/calomp_sciara-fv2, compiled unmodified from
 * its sources): the example's main() with the paths, step count and
 * active-cells switch taken from the command line, and the final state
 * written as raw little-endian doubles instead of GIS text files.
 * Test infrastructure only.
 *
 *   sciara_ref <config prefix> <steps> <active 0|1> <output file>
 * reads <prefix>_000000000000{.cfg,_Morphology.stt,_Vents.stt,
 * _EmissionRate.txt} and writes Sz, Slt, St, Msl (rows*cols doubles each),
 * then the step count reached and the active-cell count as two doubles.
 */
#include <stdio.h>
#include <string.h>

#include "Sciara.h"
#include "io.h"

Sciara* sciara;
int active;

int main(int argc, char** argv)
{
    if (argc != 5) {
        fprintf(stderr, "usage: %s prefix steps active out\n", argv[0]);
        return 2;
    }
    int steps = atoi(argv[2]);
    active = atoi(argv[3]);
    char path[1024];
    char dem[1200];
    snprintf(path, sizeof(path), "%s", argv[1]);
    snprintf(dem, sizeof(dem), "%s_000000000000_Morphology.stt", argv[1]);
    initSciara(dem, steps);
    if (!loadConfiguration(path, sciara)) {
        fprintf(stderr, "cannot load configuration\n");
        return 1;
    }
    runSciara();
    const size_t n = (size_t)sciara->rows * sciara->cols;
    FILE* f = fopen(argv[4], "wb");
    if (!f)
        return 1;
    fwrite(sciara->substates->Sz->current, sizeof(double), n, f);
    fwrite(sciara->substates->Slt->current, sizeof(double), n, f);
    fwrite(sciara->substates->St->current, sizeof(double), n, f);
    fwrite(sciara->substates->Msl->current, sizeof(double), n, f);
    double tail[2] = {(double)sciara->run->step, (double)sciara->model->A.size_current};
    fwrite(tail, sizeof(double), 2, f);
    fclose(f);
    return 0;
}
