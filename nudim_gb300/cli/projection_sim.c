/*
 * projection_sim.c -- drop-in `projection_sim` command line on the GB300
 * engine.  Options, messages and files follow src/projection_sim.c:96-247:
 * the density file holds nx*ny*nz numbers in [z][y][x] order, and
 * ./files/prj-<j>.txt receives np*nz values "%f" per tilt.
 *
 * All three methods run on the GPU.  2D1D: nudim_project_2d1d.  3D samples
 * the same 3D transform at the same nodes with a 3D NFFT (:409-514); it runs
 * as 2D1D, whose Z-FFT + 2D NFFT is that transform factorised along the
 * uniform Z axis (equal to the NFFT's accuracy).  DFT: nudim_project_dft, the
 * reference's exact sums with its truncated PI.  An unknown method name, which
 * the reference leaves undefined (:229-242), is rejected.  Noise uses the
 * library's seeded Gaussian generator (--seed, an addition; default
 * 0), not GSL's sampler.
 */
#include <getopt.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "nudim.h"
#include "textio.h"

static void show_help(const char *s)
{
    printf("\nSyntax: %s [options]\n\n", s);
    printf("Purpose: Simulate serials of tomograms from 3D density arranged in dimensions nx*ny*nz.\n"
           "         To be noted, rotation axes is along direction Z, perpendicular to paper. X is horizontal while Y is vertical.\n"
           "         And rotation angle is between X direction and incident rays.\n"
           "         Thereby, the size of each projection is np*nz.\n"
           "\n"
           "-h, --help                    Display this help message.\n"
           "\n"
           "-i, --infile=<file>           File from which to get the 3D density.\n"
           "    --nx=<nx>                 X dimension.\n"
           "    --ny=<ny>                 Y dimension.\n"
           "    --nz=<nz>                 Z dimension.\n"
           "-p, --pad=<np>                Dimension of projection in XY plane.\n"
           "    --max=<maximum gama>.     Maximum angle of tomograms for simulation.\n"
           "    --min=<minimum gama>.     Minimum angle of tomograms for simulation.\n"
           "-t, --interval=<delta angle>. Angular sampling interval.\n"
           "    --noise.                  Add noise to tomograms.\n"
           "    --snr=<value>.            Signal to noise level.\n"
           "-m  --method=<2D1D/3D/DFT>.   Use 2D NFFT + 1D FFT (default) or 3D NFFT (slow) or Discrete Fourier transform.\n"
           "    --seed=<n>.               Seed of the noise generator.\n"
           "    --device=<n>.             CUDA device.\n"
           "\n");
}

int main(int argc, char *argv[])
{
    int c;
    char *infile = NULL, *method = NULL, *rval;
    double interval = -1, gam_max = 100, gam_min = 100, snr = -1;
    int nx = -1, ny = -1, nz = -1, np = -1, config_noise = 0, device = 0;
    unsigned long seed = 0;
    const struct option longopts[] = {
        {"help", 0, NULL, 'h'}, {"infile", 1, NULL, 'i'}, {"pad", 1, NULL, 'p'},
        {"interval", 1, NULL, 't'}, {"method", 1, NULL, 'm'}, {"nx", 1, NULL, 2},
        {"ny", 1, NULL, 3}, {"nz", 1, NULL, 4}, {"max", 1, NULL, 5}, {"min", 1, NULL, 6},
        {"snr", 1, NULL, 7}, {"noise", 0, NULL, 8}, {"seed", 1, NULL, 20},
        {"device", 1, NULL, 21}, {0, 0, NULL, 0}};
    while ((c = getopt_long(argc, argv, "hi:p:t:m:", longopts, NULL)) != -1) {
        switch (c) {
        case 'h': show_help(argv[0]); return 0;
        case 'i': infile = strdup(optarg); break;
        case 'p':
            np = strtol(optarg, &rval, 10);
            if (*rval != '\0') { fprintf(stderr, "Invalid X dimension!\n"); return 1; }
            break;
        case 't':
            interval = strtod(optarg, &rval);
            if (*rval != '\0') { fprintf(stderr, "Invalid angular sampling interval!\n"); return 1; }
            break;
        case 'm': method = strdup(optarg); break;
        case 2:
            nx = strtol(optarg, &rval, 10);
            if (*rval != '\0') { fprintf(stderr, "Invalid X dimension!\n"); return 1; }
            break;
        case 3:
            ny = strtol(optarg, &rval, 10);
            if (*rval != '\0') { fprintf(stderr, "Invalid Y dimension!\n"); return 1; }
            break;
        case 4:
            nz = strtol(optarg, &rval, 10);
            if (*rval != '\0') { fprintf(stderr, "Invalid Z dimension!\n"); return 1; }
            break;
        case 5:
            gam_max = strtod(optarg, &rval);
            if (*rval != '\0') { fprintf(stderr, "Invalid maximum collecting angle!\n"); return 1; }
            break;
        case 6:
            gam_min = strtod(optarg, &rval);
            if (*rval != '\0') { fprintf(stderr, "Invalid minimum collecting angle!\n"); return 1; }
            break;
        case 7:
            snr = strtod(optarg, &rval);
            if (*rval != '\0') { fprintf(stderr, "Invalid signal to noise ratio!\n"); return 1; }
            break;
        case 8: config_noise = 1; break;
        case 20: seed = strtoul(optarg, &rval, 10); break;
        case 21: device = strtol(optarg, &rval, 10); break;
        default: return 1;
        }
    }
    if (infile == NULL) {
        fprintf(stderr, "You need to provide 3D density with --infile.\n");
        return 1;
    }
    if (nx < 0 || ny < 0 || nz < 0) {
        fprintf(stderr, "You need to provide valid dimensions with --nx, --ny, --nz.\n");
        return 1;
    }
    if (np < 0) {
        fprintf(stderr, "You need to provide valid projection dimension in XY plane with --pad.\n");
        return 1;
    }
    if (interval < 0) {
        fprintf(stderr, "You need to provide valid angular sampling interval with --interval.\n");
        return 1;
    }
    if (gam_max < -90 || gam_max > 90 || gam_min < -90 || gam_max > 90) {
        fprintf(stderr, "You need to provide valid scope of tomogram angles (-90,90] with --max, --min.\n");
        return 1;
    }
    int exact = 0;
    if (method == NULL) {
        fprintf(stderr, "You didn't specify simulating method, so I'm  using"
                        " the 2D1D method, which is fastest.\n");
    } else if (strcmp(method, "DFT") == 0) {
        exact = 1;
    } else if (strcmp(method, "2D1D") != 0 && strcmp(method, "3D") != 0) {
        fprintf(stderr, "Unknown simulating method %s (2D1D, 3D or DFT).\n", method);
        return 1;
    }
    if (config_noise && snr < 0) {
        fprintf(stderr, "You must provide valid signal to noise ratio with --snr or delete --noise.\n");
        return 1;
    }
    size_t V = (size_t)nx * ny * nz;
    double *dens = (double *)malloc(sizeof(double) * (V ? V : 1));
    if (nudim_read_numbers(infile, dens, V)) {
        fprintf(stderr, "Error : Data file %s doesn't exist!\n ", infile);
        return 1;
    }
    int ns = (int)((gam_max - gam_min) / interval + 0.5) + 1;
    size_t per = (size_t)np * nz;
    double *proj = (double *)malloc(sizeof(double) * per * (ns > 0 ? ns : 1));
    nudim_ctx *ctx;
    int rc = nudim_ctx_create(device, 0, &ctx);
    if (!rc)
        rc = (exact ? nudim_project_dft : nudim_project_2d1d)(ctx, dens, nx, ny, nz, np, gam_min,
                                                              gam_max, interval,
                                                              config_noise ? snr : 0.0, seed,
                                                              proj, per * ns);
    if (rc) {
        fprintf(stderr, "projection_sim failed (%d): %s\n", rc, nudim_last_error());
        return 1;
    }
    for (int j = 0; j < ns; j++) {
        char filename[1024];
        snprintf(filename, 1023, "./files/prj-%i.txt", j);
        if (nudim_write_numbers(filename, proj + (size_t)j * per, per, "%f")) return 1;
    }
    nudim_ctx_destroy(ctx);
    free(dens);
    free(proj);
    return 0;
}
