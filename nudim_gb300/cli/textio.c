/* textio.c -- reading and writing the reference's one-number-per-line text
 * files (src/reconstruction.c:341-358, 531-540, 706-719;
 * src/projection_sim.c:257-266, 396-403). */
#include "textio.h"

#include <stdio.h>
#include <stdlib.h>
#include <string.h>

int nudim_read_numbers(const char *path, double *out, size_t n)
{
    FILE *fp = fopen(path, "rb");
    if (!fp) {
        fprintf(stderr, "Error : file %s doesn't exist!\n", path);
        return -1;
    }
    fseek(fp, 0, SEEK_END);
    long sz = ftell(fp);
    fseek(fp, 0, SEEK_SET);
    char *buf = (char *)malloc((size_t)(sz > 0 ? sz : 0) + 1);
    if (!buf) {
        fclose(fp);
        return -2;
    }
    size_t got = fread(buf, 1, (size_t)(sz > 0 ? sz : 0), fp);
    fclose(fp);
    buf[got] = '\0';
    char *p = buf, *end;
    size_t i = 0;
    for (; i < n; i++) {
        double v = strtod(p, &end);
        if (end == p) break;
        out[i] = v;
        p = end;
    }
    free(buf);
    if (i != n) {
        fprintf(stderr, "Error : file %s holds %zu values, %zu expected!\n", path, i, n);
        return -2;
    }
    return 0;
}

int nudim_write_numbers(const char *path, const double *v, size_t n, const char *fmt)
{
    FILE *fp = fopen(path, "w");
    if (!fp) {
        fprintf(stderr, "Error : cannot write %s\n", path);
        return -1;
    }
    static char buf[1 << 20];
    setvbuf(fp, buf, _IOFBF, sizeof buf);
    char line[64];
    for (size_t i = 0; i < n; i++) {
        int k = snprintf(line, sizeof line, fmt, v[i]);
        line[k] = '\n';
        fwrite(line, 1, (size_t)k + 1, fp);
    }
    int rc = fclose(fp);
    return rc ? -1 : 0;
}
