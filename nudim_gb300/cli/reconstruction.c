/*
 * reconstruction.c -- drop-in `reconstruction` / `reconstruction_parallel`
 * command line on the GB300 engine (libnudim.so).
 *
 * Same options, validation messages, input files and output files as
 * src/reconstruction.c (NUDIM_CLI_VARIANT=0) and
 * src/reconstruction-parallel.c (NUDIM_CLI_VARIANT=1).  The parallel variant
 * keeps its behavioural deltas (diffusion lambda 0.4, TV without the height
 * window, height window centred at np/2, gradient-magnitude dumps at
 * iteration 0, "-parallel" file names, total-time line) and runs on one GPU:
 * MPI ranks do not exist here, so no rank-count check applies.
 *
 * Options added here (no collision with the reference's):
 *   --precision=FP64|MIXED   arithmetic form (default FP64)
 *   --correct=<k>            MIXED: FP64 corrective iteration every k (0: off)
 *   --device=<n>             CUDA device (default 0)
 *   --fill=<file>            values for the unknown samples with --random
 *   --autotune               time the NFFT plan candidates once, keep the fastest
 */
#include <getopt.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "nudim.h"
#include "textio.h"

#ifndef NUDIM_CLI_VARIANT
#define NUDIM_CLI_VARIANT 0
#endif

static void show_help(const char *s)
{
    printf("\nSyntax: %s [options]\n\n", s);
    printf("Purpose: Reconstruct 3D object from series of equally-angled tomograms.\n"
           "         To be noted, rotation axes is along direction Z, perpendicular to paper. X is horizontal while Y is vertical.\n"
           "         And rotation angle is between X direction and incident rays.\n"
           "         Thereby, the size of each projection is nx*nz , and nx is first ordered, namely projection[nz][nx].\n"
           "\n"
           "-h, --help                    Display this help message.\n"
           "\n"
           "    --prefix=<prefix name>.   Prefix name of series of projections.\n"
           "    --nx=<nx>                 X dimension size of projection.\n"
           "    --nz=<nz>                 Z dimension size of projection.\n"
           "-p, --pad=<np>                Padded size along radial direction, which must be at least larger than nx to achieve oversampling.\n"
           "    --max=<maximum gama>.     Maximum angle of tomograms.\n"
           "    --min=<minimum gama>.     Minimum angle of tomograms.\n"
           "-t, --interval=<delta angle>. Angular sampling interval.\n"
           "    --padangle=<pad interval>.Filling unknown region every padangle, which should be divided by the above interval.\n"
           "    --weight.                 Add weight to fourier slices to compensate for uneven sampling density among different frequencies.\n"
           "    --denoise.                Filtering 3D density at each iteration.\n"
           "    --method=<DIFFUSION/TV>.  Use anisotropic diffusion or total variation to denoise 3D density.\n"
           "    --nhio=<nhio>.            Number of HIO iterations.\n"
           "    --ner=<ner>.              Number of ER iterations.\n"
#if NUDIM_CLI_VARIANT == 0
           "    --height=<nheight>.       Sample height for constraint (in pixel).\n"
           "    --center=<ncenter>.       Sample center for constraint (in pixel).\n"
#else
           "    --height.                 Sample height for constraint.\n"
#endif
           "    --random.                 Padding unknown projections with randoms or zeros.\n"
           "    --print.                  Print out R factor with each cycle of iteration.\n"
           "    --precision=<FP64/MIXED>. Arithmetic form on the GPU (default FP64).\n"
           "    --correct=<k>.            MIXED form: FP64 corrective iteration every k iterations.\n"
           "    --device=<n>.             CUDA device.\n"
           "    --fill=<file>.            Values of the unknown samples used with --random.\n"
           "    --autotune.               Time the NFFT plan candidates once, keep the fastest.\n"
           "\n");
}

static double now_s(void)
{
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return ts.tv_sec + 1e-9 * ts.tv_nsec;
}

/* denoise.c:381-402 (debug dump of the parallel variant) */
static void grad_mag(const double *img, double *out, int NZ, int NY, int NX)
{
    size_t V = (size_t)NZ * NY * NX;
    memcpy(out, img, sizeof(double) * V);
    for (int i = 1; i < NZ - 1; i++)
        for (int j = 1; j < NY - 1; j++)
            for (int k = 1; k < NX - 1; k++) {
                size_t o = ((size_t)i * NY + j) * NX + k;
                double c = img[o], a = c - img[o - (size_t)NY * NX], b = c - img[o - NX],
                       d = c - img[o - 1];
                out[o] = sqrt(a * a + b * b + d * d);
            }
}

static int fail(const char *what, int rc)
{
    fprintf(stderr, "%s failed (%d): %s\n", what, rc, nudim_last_error());
    return 1;
}

int main(int argc, char *argv[])
{
    double t_start = now_s();
    int c;
    char *prefix = NULL, *method = NULL, *rval, *fill_path = NULL;
    double interval = -1, padangle = -1, gam_max = 100, gam_min = 100;
    int nx = -1, nz = -1, nheight = -1, ncenter = -1, np = -1, nhio = -1, ner = -1;
    int config_denoise = 0, config_random = 0, config_weight = 0, config_print = 0,
        config_height = 0;
    int precision = NUDIM_FP64, correct = 0, device = 0, denoise_m = -1, autotune = 0;

    const struct option longopts[] = {
        {"help", 0, NULL, 'h'},       {"pad", 1, NULL, 'p'},      {"interval", 1, NULL, 't'},
        {"prefix", 1, NULL, 2},       {"nx", 1, NULL, 3},         {"nz", 1, NULL, 4},
        {"max", 1, NULL, 5},          {"min", 1, NULL, 6},        {"method", 1, NULL, 7},
        {"nhio", 1, NULL, 8},         {"ner", 1, NULL, 9},        {"denoise", 0, NULL, 10},
        {"random", 0, NULL, 11},      {"print", 0, NULL, 12},     {"padangle", 1, NULL, 13},
        {"height", 1, NULL, 14},
#if NUDIM_CLI_VARIANT == 0
        {"center", 1, NULL, 15},      {"weight", 0, NULL, 16},
#else
        {"weight", 0, NULL, 16},
#endif
        {"precision", 1, NULL, 20},   {"correct", 1, NULL, 21},   {"device", 1, NULL, 22},
        {"fill", 1, NULL, 23},        {"autotune", 0, NULL, 24},  {0, 0, NULL, 0}};

    while ((c = getopt_long(argc, argv, "hp:t:", longopts, NULL)) != -1) {
        switch (c) {
        case 'h': show_help(argv[0]); return 0;
        case 'p':
            np = strtol(optarg, &rval, 10);
            if (*rval != '\0') { fprintf(stderr, "Invalid X dimension!\n"); return 1; }
            break;
        case 't':
            interval = strtod(optarg, &rval);
            if (*rval != '\0') { fprintf(stderr, "Invalid angular sampling interval!\n"); return 1; }
            break;
        case 2: prefix = strdup(optarg); break;
        case 3:
            nx = strtol(optarg, &rval, 10);
            if (*rval != '\0') { fprintf(stderr, "Invalid X dimension!\n"); return 1; }
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
        case 7: method = strdup(optarg); break;
        case 8:
            nhio = strtol(optarg, &rval, 10);
            if (*rval != '\0') { fprintf(stderr, "Invalid number of HIO!\n"); return 1; }
            break;
        case 9:
            ner = strtol(optarg, &rval, 10);
            if (*rval != '\0') { fprintf(stderr, "Invalid number of ER!\n"); return 1; }
            break;
        case 10: config_denoise = 1; break;
        case 11: config_random = 1; break;
        case 12: config_print = 1; break;
        case 13:
            padangle = strtod(optarg, &rval);
            if (*rval != '\0') { fprintf(stderr, "Invalid padded angular interval!\n"); return 1; }
            break;
        case 14:
            config_height = 1;
            nheight = strtol(optarg, &rval, 10);
            if (*rval != '\0') { fprintf(stderr, "Invalid sample height!\n"); return 1; }
            break;
        case 15:
            config_height = 1;
            ncenter = strtol(optarg, &rval, 10);
            if (*rval != '\0') { fprintf(stderr, "Invalid sample center!\n"); return 1; }
            break;
        case 16: config_weight = 1; break;
        case 20:
            if (strcmp(optarg, "FP64") == 0) precision = NUDIM_FP64;
            else if (strcmp(optarg, "MIXED") == 0) precision = NUDIM_MIXED;
            else { fprintf(stderr, "Invalid precision (FP64 or MIXED)!\n"); return 1; }
            break;
        case 21:
            correct = strtol(optarg, &rval, 10);
            if (*rval != '\0' || correct < 0) { fprintf(stderr, "Invalid correction period!\n"); return 1; }
            break;
        case 22:
            device = strtol(optarg, &rval, 10);
            if (*rval != '\0') { fprintf(stderr, "Invalid device!\n"); return 1; }
            break;
        case 23: fill_path = strdup(optarg); break;
        case 24: autotune = 1; break;
        default: return 1;
        }
    }

    /* src/reconstruction.c:245-293 (parallel: reconstruction-parallel.c:251-300) */
    if (prefix == NULL) {
        fprintf(stderr, "You need to provide prefix name of tomogram files with --prefix.\n");
        return 1;
    }
    if (nx < 0 || nz < 0) {
        fprintf(stderr, "You need to provide valid projection size with --nx, --nz.\n");
        return 1;
    }
    if (np < 0) {
        fprintf(stderr, "You need to provide valid projection dimension in XY plane with --pad.\n");
        return 1;
    }
    if (nhio < 0) { fprintf(stderr, "You need to provide valid nhio with --nhio.\n"); return 1; }
    if (ner < 0) { fprintf(stderr, "You need to provide valid ner with --ner.\n"); return 1; }
    if (interval < 0) {
        fprintf(stderr, "You need to provide valid angular sampling interval with --interval.\n");
        return 1;
    }
    if (padangle < 0 || interval / padangle - (int)(interval / padangle + 0.1) > 1e-5) {
        fprintf(stderr, "You need to provide valid padded angular sampling interval with --padangle.\n");
        return 1;
    }
    if (gam_max < -90 || gam_max > 90 || gam_min < -90 || gam_max > 90) {
        fprintf(stderr, "You need to provide valid scope of tomogram angles (-90,90] with --max, --min.\n");
        return 1;
    }
    if (config_denoise && method == NULL) {
        fprintf(stderr, "You must provide valid denoising method or delete --denoise.\n");
        return 1;
    }
#if NUDIM_CLI_VARIANT == 0
    if (config_height && (nheight <= 0 || ncenter <= 0)) {
        fprintf(stderr, "You must provide valid both sample height and center with --height and --center.\n");
        return 1;
    }
#else
    if (config_height && nheight <= 0) {
        fprintf(stderr, "You must provide valid sample height --height.\n");
        return 1;
    }
#endif
    if (method != NULL) {
        if (strcmp(method, "DIFFUSION") == 0) denoise_m = NUDIM_DENOISE_DIFFUSION;
        else if (strcmp(method, "TV") == 0) denoise_m = NUDIM_DENOISE_TV;
        else if (config_denoise) {
            fprintf(stderr, "Unknown denoising method %s (DIFFUSION or TV).\n", method);
            return 1;
        }
        free(method);
    }

    nudim_job_desc d;
    memset(&d, 0, sizeof d);
    d.nx = nx; d.nz = nz; d.np = np;
    d.gam_min = gam_min; d.gam_max = gam_max; d.interval = interval; d.padangle = padangle;
    d.nhio = nhio; d.ner = ner;
    d.denoise = config_denoise ? denoise_m : NUDIM_DENOISE_NONE;
    d.weight = config_weight; d.random = config_random;
    d.height = config_height; d.nheight = nheight; d.ncenter = ncenter;
    d.variant = NUDIM_CLI_VARIANT;
    d.precision = precision; d.cgnr_iters = 10; d.correct_every = correct;

    int nslices = (int)((gam_max - gam_min) / interval + 0.5) + 1;
    if (nslices <= 0 || nx == 0 || nz == 0) {
        fprintf(stderr, "Empty tilt series.\n");
        return 1;
    }
    size_t per = (size_t)nx * nz;
    double *proj = (double *)malloc(sizeof(double) * per * nslices);
    if (!proj) { fprintf(stderr, "Out of host memory.\n"); return 1; }
    for (int j = 0; j < nslices; j++) {
        char filename[1024];
        snprintf(filename, 1023, "./files/%s-%i.txt", prefix, j);
        if (nudim_read_numbers(filename, proj + (size_t)j * per, per)) return 1;
    }
    free(prefix);

    nudim_ctx *ctx;
    nudim_job *job;
    int rc = nudim_ctx_create(device, autotune ? NUDIM_CTX_AUTOTUNE : 0u, &ctx);
    if (rc) return fail("nudim_ctx_create", rc);
    rc = nudim_job_create(ctx, &d, &job);
    if (rc) return fail("nudim_job_create", rc);
    if (config_random && fill_path) {
        FILE *fp = fopen(fill_path, "r");
        size_t cnt = 0;
        double v;
        if (!fp) { fprintf(stderr, "Error : file %s doesn't exist!\n", fill_path); return 1; }
        while (fscanf(fp, "%le", &v) == 1) cnt++;
        fclose(fp);
        double *fill = (double *)malloc(sizeof(double) * (cnt ? cnt : 1));
        if (nudim_read_numbers(fill_path, fill, cnt)) return 1;
        rc = nudim_job_import_fill(job, fill, cnt);
        free(fill);
        if (rc) return fail("nudim_job_import_fill", rc);
    }
    rc = nudim_job_set_projections(job, proj, per * nslices);
    free(proj);
    if (rc) return fail("nudim_job_set_projections", rc);

    size_t V = (size_t)np * np * nz;
    double *vol = (double *)malloc(sizeof(double) * V);
    rc = nudim_job_get_initial_volume(job, vol, V);
    if (rc) return fail("nudim_job_get_initial_volume", rc);
    if (nudim_write_numbers(NUDIM_CLI_VARIANT ? "recovered-0-parallel.txt" : "recovered-0.txt",
                            vol, V, "%le"))
        return 1;

    int dump_nn = NUDIM_CLI_VARIANT ? 0 : 100;
    double *before = NULL, *after = NULL;
    if (config_denoise && dump_nn < nhio + ner) {
        before = (double *)malloc(sizeof(double) * V);
        after = (double *)malloc(sizeof(double) * V);
        nudim_job_set_denoise_dump(job, dump_nn, before, after);
    }
    int total = nhio + ner;
    if (config_print || before) {
        double *rh = (double *)malloc(sizeof(double) * (total ? total : 1));
        for (int nn = 0; nn < total; nn++) {
            rc = nudim_step(ctx, &job, 1, 1);
            if (rc) return fail("nudim_step", rc);
            if (config_print) {
                int cnt = 0;
                rc = nudim_job_get_rfactor(job, rh, total, &cnt);
                if (rc) return fail("nudim_job_get_rfactor", rc);
                printf("Iteration: %d Measured Residual: %f\n", nn, rh[nn]);
            }
            if (before && nn == dump_nn) {
                nudim_ctx_sync(ctx);
                if (NUDIM_CLI_VARIANT) {
                    grad_mag(before, vol, nz, np, np);
                    nudim_write_numbers("grad_before.txt", vol, V, "%f");
                    grad_mag(after, vol, nz, np, np);
                    nudim_write_numbers("grad_after.txt", vol, V, "%f");
                } else {
                    nudim_write_numbers("grad_before.txt", before, V, "%f");
                    nudim_write_numbers("grad_after.txt", after, V, "%f");
                }
            }
        }
        free(rh);
    } else {
        rc = nudim_step(ctx, &job, 1, total);
        if (rc) return fail("nudim_step", rc);
    }
    size_t Vc = (size_t)nx * nx * nz;
    rc = nudim_job_get_volume(job, vol, Vc, 1);
    if (rc) return fail("nudim_job_get_volume", rc);
    if (nudim_write_numbers(NUDIM_CLI_VARIANT ? "recovered-parallel.txt" : "recovered.txt", vol,
                            Vc, "%f"))
        return 1;
    free(vol);
    free(before);
    free(after);
    nudim_job_destroy(job);
    nudim_ctx_destroy(ctx);
    if (NUDIM_CLI_VARIANT) printf("Total time used : %f seconds.\n", now_s() - t_start);
    return 0;
}
