/* textio.h -- the reference's text formats: one ASCII number per line. */
#ifndef NUDIM_TEXTIO_H
#define NUDIM_TEXTIO_H
#include <stddef.h>

/* Read exactly n numbers (any whitespace-separated %le-readable text) from
 * path into out.  Returns 0, or -1 (missing file) / -2 (short or bad file)
 * with a message on stderr. */
int nudim_read_numbers(const char *path, double *out, size_t n);

/* Write n numbers, one per line, with printf format fmt ("%le" or "%f"). */
int nudim_write_numbers(const char *path, const double *v, size_t n, const char *fmt);

#endif
