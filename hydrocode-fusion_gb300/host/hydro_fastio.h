/*
 * hydro_fastio.h -- multi-threaded readers and writers of the drivers' data
 * files, and a binary FP64 format beside the reference's text.
 *
 * The reference reads initial data with getc one character at a time
 * (src/file_io/io_control.c:163-261) and writes %.10g text with one fprintf
 * per value (src/file_io/file_2D_out.c:55-101); at 4096^2 both take seconds to
 * minutes of one core.  The functions here produce the same numbers and the
 * same bytes on several threads:
 *   - hio_read_table: the numbers of a whitespace-separated text file, with
 *     the reference reader's character rules, line/column counting, strtod
 *     conversion and error messages;
 *   - hio_write_text: rows of "%.10g\t" values, formatted by several threads
 *     and written in order, byte for byte what one fprintf per value writes;
 *   - a binary file of FP64 planes (header, snapshot times, planes in the text
 *     files' row order) and its reader.
 * Threads: HYDRO_IO_THREADS, else the online processors (at most 16).
 */
#ifndef HYDRO_FASTIO_H
#define HYDRO_FASTIO_H

#include <stdio.h>

/* Value of row r, column c of one plane (2D text: row = y index, column = x index). */
typedef double (*hio_value_fn)(const void *ctx, int r, int c);

/* Threads the I/O functions use: HYDRO_IO_THREADS when set (>= 1), else the
 * online processors capped at 16. */
int hio_threads(void);

/* Reads every number of a text file.  On success returns 0 and sets *lines
 * (lines holding at least one number), *columns (numbers on the first such
 * line; every such line must hold as many when check_columns != 0), *count
 * (all numbers) and *data (malloc'd, file order).  Errors print the
 * reference reader's message and return 1 (illegal character), 2 (unequal
 * columns), 3 (an entry strtod does not take whole, or out of range),
 * 4 (cannot open/read), 5 (memory).  Unlike the reference, a last number
 * not followed by whitespace is read (the reference leaves it unset). */
int hio_read_table(const char *path, int check_columns, int *lines, int *columns, long long *count, double **data);

/* Writes rows x cols values as "%.10g\t" each, rows ended by "\n". */
int hio_write_text(FILE *fp, int rows, int cols, hio_value_fn f, const void *ctx);

/* Binary FP64 file: "HCFBIN01", then int32 ndim, n_x, n_y, nsnap, 0 (little
 * endian), nsnap float64 times, then nsnap planes of n_y rows x n_x float64
 * (row = y index, as the text files; 1D files have n_y = 1). */
FILE *hio_bin_create(const char *path, int ndim, int n_x, int n_y, int nsnap, const double *times);
int hio_bin_plane(FILE *fp, int rows, int cols, hio_value_fn f, const void *ctx);
/* Reads a binary file: header fields, *times (malloc'd, nsnap) and *data
 * (malloc'd, nsnap*n_y*n_x).  0, or 4 (I/O / format) or 5 (memory). */
int hio_bin_read(const char *path, int *ndim, int *n_x, int *n_y, int *nsnap, double **times, double **data);

#endif
