/* mrc2prj -- convert an MRC tilt series into the projection text files the
 * reconstruction executables read (./files/<prefix>-<j>.txt, one "%f" value
 * per line, [row][column] order).  Host-only data preparation, standing in
 * for the reference's example converter (examples/exp/mrcread.c with
 * examples/exp/mrcfile.c):
 *
 *   - the header's first words give nx, ny, nz and the mode; slice data start
 *     at byte 1024 as in the reference reader (--ext-header adds the
 *     extended-header length, header word 23, for files that carry one);
 *   - modes 0 (unsigned byte), 1 (signed short), 2 (float) as the reference,
 *     and 6 (unsigned short); little-endian host order, as the reference;
 *   - per slice, optionally: a cyclic shift left by --shift-x columns, the
 *     columns that wrap moving up by --shift-y rows (the reference's fixed
 *     61 and 1); --invert writes max - v + min with max/min over the slice
 *     (initial extrema -1e5 and 1e5, as the reference); --skip-first drops
 *     slice 0; --reverse numbers slice k as nz - 1 - k.
 *
 * The reference example's conversion is
 *   mrc2prj --in BBa.ali --shift-x 61 --shift-y 1 --invert --skip-first --reverse
 */
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/stat.h>

#include "textio.h"

static void usage(void)
{
    fprintf(stderr,
            "usage: mrc2prj --in FILE [--prefix prj] [--shift-x S] [--shift-y T] [--invert]\n"
            "               [--skip-first] [--reverse] [--ext-header]\n");
}

static int32_t word(const unsigned char *h, int i)
{
    int32_t v;
    memcpy(&v, h + 4 * i, 4);
    return v;
}

int main(int argc, char **argv)
{
    const char *in = NULL, *prefix = "prj";
    int sx = 0, sy = 0, invert = 0, skip_first = 0, reverse = 0, ext = 0;
    for (int a = 1; a < argc; a++) {
        if (!strcmp(argv[a], "--in") && a + 1 < argc) in = argv[++a];
        else if (!strcmp(argv[a], "--prefix") && a + 1 < argc) prefix = argv[++a];
        else if (!strcmp(argv[a], "--shift-x") && a + 1 < argc) sx = atoi(argv[++a]);
        else if (!strcmp(argv[a], "--shift-y") && a + 1 < argc) sy = atoi(argv[++a]);
        else if (!strcmp(argv[a], "--invert")) invert = 1;
        else if (!strcmp(argv[a], "--skip-first")) skip_first = 1;
        else if (!strcmp(argv[a], "--reverse")) reverse = 1;
        else if (!strcmp(argv[a], "--ext-header")) ext = 1;
        else {
            usage();
            return 1;
        }
    }
    if (!in) {
        usage();
        return 1;
    }
    FILE *fp = fopen(in, "rb");
    if (!fp) {
        fprintf(stderr, "Error : file %s doesn't exist!\n", in);
        return 1;
    }
    unsigned char h[1024];
    if (fread(h, 1, sizeof h, fp) != sizeof h) {
        fprintf(stderr, "Error : %s is shorter than an MRC header\n", in);
        fclose(fp);
        return 1;
    }
    const int nx = word(h, 0), ny = word(h, 1), nz = word(h, 2), mode = word(h, 3);
    const long start = 1024 + (ext ? (long)word(h, 23) : 0);
    int psize = mode == 0 ? 1 : mode == 1 || mode == 6 ? 2 : mode == 2 ? 4 : 0;
    if (nx <= 0 || ny <= 0 || nz <= 0 || !psize || start < 1024) {
        fprintf(stderr, "Error : unsupported MRC file (nx %d ny %d nz %d mode %d)\n", nx, ny, nz,
                mode);
        fclose(fp);
        return 1;
    }
    printf("Data Dimension: %d %d %d\n", nx, ny, nz);
    printf("Data type (Mode): %d\n", mode);
    const size_t per = (size_t)nx * ny;
    unsigned char *raw = (unsigned char *)malloc(per * psize);
    float *slc = (float *)malloc(per * sizeof(float));
    double *out = (double *)malloc(per * sizeof(double));
    if (!raw || !slc || !out) {
        fclose(fp);
        return 1;
    }
    mkdir("files", 0755);
    int rc = 0;
    for (int k = skip_first ? 1 : 0; k < nz && !rc; k++) {
        if (fseek(fp, start + (long)k * (long)(per * psize), SEEK_SET) ||
            fread(raw, psize, per, fp) != per) {
            fprintf(stderr, "Error : %s ends inside slice %d\n", in, k);
            rc = 1;
            break;
        }
        for (size_t i = 0; i < per; i++) {
            if (mode == 0) slc[i] = (float)raw[i];
            else if (mode == 1) {
                int16_t v;
                memcpy(&v, raw + 2 * i, 2);
                slc[i] = (float)v;
            } else if (mode == 6) {
                uint16_t v;
                memcpy(&v, raw + 2 * i, 2);
                slc[i] = (float)v;
            } else {
                memcpy(&slc[i], raw + 4 * i, 4);
            }
        }
        double mx = -100000, mn = 100000;
        for (size_t i = 0; i < per; i++) {
            if (slc[i] > mx) mx = slc[i];
            if (slc[i] < mn) mn = slc[i];
        }
        /* shifted image: column i goes to (i - sx) mod nx; the wrapped
           columns (i < sx) also move to row (j - sy) mod ny */
        for (int j = 0; j < ny; j++)
            for (int i = 0; i < nx; i++) {
                int col = ((i - sx) % nx + nx) % nx;
                int row = i < sx ? ((j - sy) % ny + ny) % ny : j;
                float v = slc[(size_t)j * nx + i];
                out[(size_t)row * nx + col] = invert ? mx - v + mn : (double)v;
            }
        if (invert) printf("%f %f \n", mx, mn);
        char name[1100];
        snprintf(name, sizeof name, "./files/%s-%d.txt", prefix, reverse ? nz - 1 - k : k);
        if (nudim_write_numbers(name, out, per, "%f")) rc = 1;
    }
    free(raw);
    free(slc);
    free(out);
    fclose(fp);
    return rc;
}
