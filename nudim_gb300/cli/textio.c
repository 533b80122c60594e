/* textio.c -- reading and writing the reference's one-number-per-line text
 * files (src/reconstruction.c:341-358, 531-540, 706-719;
 * src/projection_sim.c:257-266, 396-403).
 *
 * Both directions run on the host's cores: the reader splits the file at
 * whitespace, counts the numbers of every piece, then parses the pieces in
 * parallel (strtod, as a sequential reader would); the writer formats blocks
 * of values in parallel with the caller's printf format and writes them in
 * order.  The bytes read and written are those of the one-thread loops. */
#include "textio.h"

#include <ctype.h>
#include <pthread.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

enum { kMaxThreads = 16 };

static int host_threads(size_t work, size_t grain)
{
    long hw = sysconf(_SC_NPROCESSORS_ONLN);
    size_t t = work / grain;
    if (t < 1) t = 1;
    if (hw < 1) hw = 1;
    if (t > (size_t)hw) t = (size_t)hw;
    if (t > kMaxThreads) t = kMaxThreads;
    return (int)t;
}

/* ------------------------------------------------------------------ read */
struct read_piece {
    const char *beg, *end;  /* [beg, end) starts and ends at whitespace or the file ends */
    size_t count;           /* numbers in the piece */
    double *out;            /* where the piece's first number goes */
    size_t parsed;
};

static void *count_piece(void *arg)
{
    struct read_piece *p = (struct read_piece *)arg;
    size_t c = 0;
    int in = 0;
    for (const char *s = p->beg; s < p->end; s++) {
        int ws = isspace((unsigned char)*s);
        if (!ws && !in) c++;
        in = !ws;
    }
    p->count = c;
    return NULL;
}

static void *parse_piece(void *arg)
{
    struct read_piece *p = (struct read_piece *)arg;
    const char *s = p->beg;
    char *e;
    size_t i = 0;
    for (; i < p->count; i++) {
        double v = strtod(s, &e);
        if (e == s || e > p->end) break;
        p->out[i] = v;
        s = e;
    }
    p->parsed = i;
    return NULL;
}

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
    size_t len = (size_t)(sz > 0 ? sz : 0);
    char *buf = (char *)malloc(len + 1);
    if (!buf) {
        fclose(fp);
        return -2;
    }
    size_t got = fread(buf, 1, len, fp);
    fclose(fp);
    buf[got] = '\0';
    /* pieces split at whitespace, so no number straddles two */
    int nt = host_threads(got, (size_t)1 << 22);
    struct read_piece pc[kMaxThreads];
    const char *cut = buf;
    for (int k = 0; k < nt; k++) {
        const char *e = k == nt - 1 ? buf + got : buf + got * (size_t)(k + 1) / (size_t)nt;
        if (e < cut) e = cut;
        while (e < buf + got && !isspace((unsigned char)*e)) e++;
        pc[k].beg = cut;
        pc[k].end = e;
        cut = e;
    }
    pthread_t th[kMaxThreads];
    for (int k = 1; k < nt; k++) pthread_create(&th[k], NULL, count_piece, &pc[k]);
    count_piece(&pc[0]);
    for (int k = 1; k < nt; k++) pthread_join(th[k], NULL);
    size_t total = 0;
    for (int k = 0; k < nt; k++) {
        pc[k].out = out + (total < n ? total : n);
        if (total + pc[k].count > n) pc[k].count = total < n ? n - total : 0;
        total += pc[k].count;
    }
    for (int k = 1; k < nt; k++) pthread_create(&th[k], NULL, parse_piece, &pc[k]);
    parse_piece(&pc[0]);
    for (int k = 1; k < nt; k++) pthread_join(th[k], NULL);
    size_t i = 0;
    int bad = 0;
    for (int k = 0; k < nt; k++) {
        i += pc[k].parsed;
        if (pc[k].parsed != pc[k].count) {
            bad = 1;
            break;
        }
    }
    free(buf);
    if (bad || i != n) {
        fprintf(stderr, "Error : file %s holds %zu values, %zu expected!\n", path, i, n);
        return -2;
    }
    return 0;
}

/* ------------------------------------------------------------------ write */
enum { kBlock = 1 << 20 };  /* values formatted per thread and round */

struct write_piece {
    const double *v;
    size_t n;
    const char *fmt;
    char *text;
    size_t bytes;
};

static void *format_piece(void *arg)
{
    struct write_piece *p = (struct write_piece *)arg;
    size_t cap = p->n * 32 + 64, k = 0;
    p->text = (char *)malloc(cap);
    if (!p->text) {
        p->bytes = 0;
        return NULL;
    }
    for (size_t i = 0; i < p->n; i++) {
        for (;;) {
            size_t room = cap - k;
            int w = snprintf(p->text + k, room, p->fmt, p->v[i]);
            if (w >= 0 && (size_t)w + 1 < room) {
                k += (size_t)w;
                p->text[k++] = '\n';
                break;
            }
            /* a long line (e.g. %f of a huge value): grow and format again */
            cap = 2 * cap + (w > 0 ? (size_t)w : 0) + 64;
            char *t = (char *)realloc(p->text, cap);
            if (!t || w < 0) {
                free(t ? t : p->text);
                p->text = NULL;
                return NULL;
            }
            p->text = t;
        }
    }
    p->bytes = k;
    return NULL;
}

int nudim_write_numbers(const char *path, const double *v, size_t n, const char *fmt)
{
    FILE *fp = fopen(path, "w");
    if (!fp) {
        fprintf(stderr, "Error : cannot write %s\n", path);
        return -1;
    }
    int nt = host_threads(n, kBlock / 4);
    int err = 0;
    for (size_t base = 0; base < n && !err;) {
        struct write_piece pc[kMaxThreads];
        pthread_t th[kMaxThreads];
        int np = 0;
        for (; np < nt && base < n; np++) {
            size_t m = n - base < kBlock ? n - base : kBlock;
            pc[np].v = v + base;
            pc[np].n = m;
            pc[np].fmt = fmt;
            pc[np].text = NULL;
            base += m;
        }
        for (int k = 1; k < np; k++) pthread_create(&th[k], NULL, format_piece, &pc[k]);
        format_piece(&pc[0]);
        for (int k = 1; k < np; k++) pthread_join(th[k], NULL);
        for (int k = 0; k < np; k++) {
            if (!pc[k].text || fwrite(pc[k].text, 1, pc[k].bytes, fp) != pc[k].bytes) err = 1;
            free(pc[k].text);
        }
    }
    int rc = fclose(fp);
    return rc || err ? -1 : 0;
}
