"""The drop-in executables' text I/O (nudim_gb300/cli/textio.c): the
parallel writer's bytes and the parallel reader's values equal those of the
one-thread loops (the reference's fprintf / fscanf one number per line), and
short or missing files fail as before."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CLI = os.path.join(os.path.dirname(HERE), "nudim_gb300", "cli")

HARNESS = r"""
#include "textio.h"
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
static void write_seq(const char *path, const double *v, size_t n, const char *fmt) {
    FILE *fp = fopen(path, "w");
    for (size_t i = 0; i < n; i++) fprintf(fp, fmt, v[i]), fputc('\n', fp);
    fclose(fp);
}
static int same(const char *a, const char *b) {
    FILE *x = fopen(a, "rb"), *y = fopen(b, "rb");
    int ca, cb, eq = 1;
    do { ca = fgetc(x); cb = fgetc(y); if (ca != cb) { eq = 0; break; } } while (ca != EOF);
    fclose(x); fclose(y);
    return eq;
}
int main(int argc, char **argv) {
    size_t n = (size_t)atol(argv[1]);
    const char *dir = argv[2];
    char pa[4096], pb[4096];
    snprintf(pa, sizeof pa, "%s/par.txt", dir);
    snprintf(pb, sizeof pb, "%s/seq.txt", dir);
    double *v = malloc((n + 8) * sizeof(double)), *r = malloc((n + 8) * sizeof(double));
    srand(11);
    for (size_t i = 0; i < n; i++)
        v[i] = ((double)rand() / RAND_MAX - 0.5) * pow(10.0, (int)(rand() % 16) - 8);
    if (n > 8) { v[1] = 1e300; v[2] = -1e-300; v[3] = 0.0; v[4] = -0.0; v[5] = 123456789.0; }
    const char *fmts[2] = {"%le", "%f"};
    for (int f = 0; f < 2; f++) {
        if (nudim_write_numbers(pa, v, n, fmts[f])) return 10;
        write_seq(pb, v, n, fmts[f]);
        if (!same(pa, pb)) return 11 + f;
        if (nudim_read_numbers(pa, r, n)) return 13;
        FILE *fp = fopen(pa, "r");
        for (size_t i = 0; i < n; i++) {
            double x;
            if (fscanf(fp, "%le", &x) != 1 || memcmp(&x, &r[i], sizeof x)) return 14;
        }
        fclose(fp);
    }
    if (nudim_read_numbers(pa, r, n + 1) != -2) return 15;
    snprintf(pb, sizeof pb, "%s/missing.txt", dir);
    if (nudim_read_numbers(pb, r, 1) != -1) return 16;
    return 0;
}
"""


@pytest.mark.parametrize("n", [1, 7, 100003, 3000017])
def test_parallel_text_io_matches_one_thread_loops(tmp_path, n):
    if shutil.which("gcc") is None:
        pytest.skip("gcc not available")
    src = tmp_path / "h.c"
    src.write_text(HARNESS)
    exe = tmp_path / "h"
    subprocess.run(["gcc", "-O2", "-I", CLI, str(src), os.path.join(CLI, "textio.c"), "-o",
                    str(exe), "-lm", "-pthread"], check=True)
    r = subprocess.run([str(exe), str(n), str(tmp_path)], capture_output=True, text=True)
    assert r.returncode == 0, (r.returncode, r.stderr)
