/*
 * hydro_fastio.c -- multi-threaded text reader/writer and the binary FP64
 * format of the drivers (hydro_fastio.h).
 *
 * Reader: the file is read into memory in one call and cut into one chunk
 * per thread at line ends.  Pass 1 (parallel) applies the reference reader's
 * character rules (src/file_io/io_control.c:163-215: a number is a run of
 * 0-9 . - e E, whitespace separates, anything else is an error) and records
 * the numbers on each line; the merge (serial, in file order) finds the
 * column count and the first error exactly where a one-pass scan would; pass
 * 2 (parallel) converts each chunk's numbers with strtod into their final
 * places (io_control.c:221-261).  Writer: row blocks are formatted with
 * snprintf("%.10g\t") by several threads into separate buffers and written
 * in row order.
 */
#define _POSIX_C_SOURCE 200809L
#include "hydro_fastio.h"

#include <ctype.h>
#include <errno.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

int hio_threads(void)
{
    const char *e = getenv("HYDRO_IO_THREADS");
    if (e) {
        int t = atoi(e);
        if (t >= 1)
            return t > 256 ? 256 : t;
    }
    long n = sysconf(_SC_NPROCESSORS_ONLN);
    if (n < 1)
        n = 1;
    return n > 16 ? 16 : (int)n;
}

static int number_char(int ch) { return ch == '-' || ch == '.' || ch == 'E' || ch == 'e' || (ch >= '0' && ch <= '9'); }

/* Runs fn(arg_k) for k < n on n threads (the calling thread takes the first). */
static int run_parallel(int n, void *(*fn)(void *), void *args, size_t arg_size)
{
    pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * (size_t)(n > 1 ? n : 1));
    int *started = (int *)calloc((size_t)(n > 1 ? n : 1), sizeof(int));
    if (!th || !started) {
        free(th);
        free(started);
        for (int k = 0; k < n; ++k)
            fn((char *)args + (size_t)k * arg_size);
        return 0;
    }
    for (int k = 1; k < n; ++k)
        started[k] = pthread_create(&th[k], NULL, fn, (char *)args + (size_t)k * arg_size) == 0;
    fn(args);
    for (int k = 1; k < n; ++k) {
        if (started[k])
            pthread_join(th[k], NULL);
        else
            fn((char *)args + (size_t)k * arg_size); /* could not start a thread: run it here */
    }
    free(th);
    free(started);
    return 0;
}

/* ---- reader ------------------------------------------------------------- */

typedef struct {
    const char *buf;
    size_t begin, end;  /* [begin, end): whole lines, the last chunk ends at the file's end */
    int last;           /* this chunk ends the file (its end is a line end too) */
    /* pass 1 */
    int *line_counts;   /* numbers on each line that holds any, in order */
    int nlines, cap;
    long long tokens;   /* numbers in the chunk (up to an illegal character) */
    int bad_char, bad_flag;  /* first illegal character (-1 none) and the number flag at it */
    int oom;
    /* pass 2 */
    double *out;        /* where this chunk's first number goes */
    long long bad_entry;  /* index within the chunk of the first entry strtod rejects (-1 none) */
} read_chunk;

static void push_line(read_chunk *c, int count)
{
    if (c->nlines == c->cap) {
        int nc = c->cap ? 2 * c->cap : 256;
        int *p = (int *)realloc(c->line_counts, sizeof(int) * (size_t)nc);
        if (!p) {
            c->oom = 1;
            return;
        }
        c->line_counts = p;
        c->cap = nc;
    }
    c->line_counts[c->nlines++] = count;
}

static void *scan_chunk(void *arg)
{
    read_chunk *c = (read_chunk *)arg;
    int flag = 0, column = 0;
    for (size_t i = c->begin; i < c->end; ++i) {
        const int ch = (unsigned char)c->buf[i];
        if (ch == '\n') {
            if (flag)
                ++column;
            flag = 0;
            if (column) {
                push_line(c, column);
                c->tokens += column;
                column = 0;
            }
        } else if (number_char(ch)) {
            flag = 1;
        } else if (!isspace(ch)) {
            c->bad_char = ch;
            c->bad_flag = flag;
            return NULL;
        } else if (flag) {
            ++column;
            flag = 0;
        }
    }
    if (c->last) {  /* the end of the file ends the last line */
        if (flag)
            ++column;
        if (column) {
            push_line(c, column);
            c->tokens += column;
        }
    }
    return NULL;
}

static void *parse_chunk(void *arg)
{
    read_chunk *c = (read_chunk *)arg;
    char number[256];
    long long j = 0;
    size_t i = c->begin;
    while (i < c->end) {
        while (i < c->end && !number_char((unsigned char)c->buf[i]))
            ++i;
        if (i >= c->end)
            break;
        size_t s = i;
        while (i < c->end && number_char((unsigned char)c->buf[i]))
            ++i;
        size_t len = i - s;
        double v = 0.0;
        int ok = len < sizeof(number);
        if (ok) {
            memcpy(number, c->buf + s, len);
            number[len] = '\0';
            char *endptr;
            errno = 0;
            v = strtod(number, &endptr);
            ok = !(errno == ERANGE || *endptr != '\0');
        }
        if (!ok) {
            c->bad_entry = j;
            return NULL;
        }
        c->out[j++] = v;
    }
    return NULL;
}

int hio_read_table(const char *path, int check_columns, int *lines, int *columns, long long *count, double **data)
{
    *lines = 0;
    *columns = 0;
    *count = 0;
    *data = NULL;
    FILE *fp = fopen(path, "rb");
    if (!fp)
        return 4;
    if (fseek(fp, 0, SEEK_END) != 0) {
        fclose(fp);
        return 4;
    }
    long size = ftell(fp);
    if (size < 0 || fseek(fp, 0, SEEK_SET) != 0) {
        fclose(fp);
        return 4;
    }
    char *buf = (char *)malloc((size_t)size + 1);
    if (!buf) {
        fclose(fp);
        return 5;
    }
    size_t got = fread(buf, 1, (size_t)size, fp);
    fclose(fp);
    if (got != (size_t)size) {
        free(buf);
        return 4;
    }
    buf[size] = '\0';

    int T = hio_threads();
    if ((long)T * 4096 > size)  /* small files: one chunk */
        T = 1;
    read_chunk *ch = (read_chunk *)calloc((size_t)T, sizeof(read_chunk));
    if (!ch) {
        free(buf);
        return 5;
    }
    size_t prev = 0;
    for (int t = 0; t < T; ++t) {
        size_t e = (t == T - 1) ? (size_t)size : (size_t)((long long)size * (t + 1) / T);
        if (t < T - 1) {
            if (e < prev)
                e = prev;
            while (e > 0 && e < (size_t)size && buf[e - 1] != '\n')
                ++e;  /* end right after a line end */
        }
        ch[t].buf = buf;
        ch[t].begin = prev;
        ch[t].end = e;
        ch[t].last = (t == T - 1);
        ch[t].bad_char = -1;
        ch[t].bad_entry = -1;
        prev = e;
    }
    run_parallel(T, scan_chunk, ch, sizeof(read_chunk));

    /* merge in file order: the first unequal line or illegal character wins */
    int rc = 0, line = 0, n_x = 0;
    long long total = 0;
    for (int t = 0; t < T && !rc; ++t) {
        if (ch[t].oom) {
            rc = 5;
            break;
        }
        for (int l = 0; l < ch[t].nlines; ++l) {
            const int col = ch[t].line_counts[l];
            if (!line)
                n_x = col;
            else if (check_columns && col != n_x) {
                printf("Error in input data file '%s', line=%d, column=%d, n_x=%d\n", path, line, col, n_x);
                rc = 2;
                break;
            }
            ++line;
        }
        if (rc)
            break;
        if (ch[t].bad_char >= 0) {
            /* the messages of flu_var_count_line (io_control.c:198) and flu_var_count (:141) */
            if (check_columns)
                printf("Input contains illigal character(ASCII=%d, flag=%d) in the file '%s', line=%d!\n",
                       ch[t].bad_char, ch[t].bad_flag, path, line);
            else
                fprintf(stderr, "Input contains illegal character(ASCII=%d, flag=%d) in the file '%s'!\n",
                        ch[t].bad_char, ch[t].bad_flag, path);
            rc = 1;
            break;
        }
        total += ch[t].tokens;
    }
    double *out = NULL;
    if (!rc && total > 0) {
        out = (double *)malloc(sizeof(double) * (size_t)total);
        if (!out)
            rc = 5;
    }
    if (!rc && total > 0) {
        long long off = 0;
        for (int t = 0; t < T; ++t) {
            ch[t].out = out + off;
            off += ch[t].tokens;
        }
        run_parallel(T, parse_chunk, ch, sizeof(read_chunk));
        long long off2 = 0;
        for (int t = 0; t < T; ++t) {
            if (ch[t].bad_entry >= 0) {
                printf("The %lldth entry in the initial data file is not a double-precision floats.\n",
                       off2 + ch[t].bad_entry + 1);
                rc = 3;
                break;
            }
            off2 += ch[t].tokens;
        }
    }
    for (int t = 0; t < T; ++t)
        free(ch[t].line_counts);
    free(ch);
    free(buf);
    if (rc) {
        free(out);
        return rc;
    }
    *lines = line;
    *columns = n_x;
    *count = total;
    *data = out;
    return 0;
}

/* ---- text writer -------------------------------------------------------- */

typedef struct {
    hio_value_fn f;
    const void *ctx;
    int r0, r1, cols;
    char *buf;
    size_t cap, len;
    int oom;
} write_task;

static void *format_rows(void *arg)
{
    write_task *w = (write_task *)arg;
    w->len = 0;
    /* "%.10g\t" is at most 17 characters (-d.ddddddddde-308 and the tab) */
    const size_t need = (size_t)(w->r1 - w->r0) * ((size_t)w->cols * 18 + 1) + 1;
    if (w->cap < need) {
        char *p = (char *)realloc(w->buf, need);
        if (!p) {
            w->oom = 1;
            return NULL;
        }
        w->buf = p;
        w->cap = need;
    }
    char *o = w->buf;
    for (int r = w->r0; r < w->r1; ++r) {
        for (int c = 0; c < w->cols; ++c)
            o += snprintf(o, 19, "%.10g\t", w->f(w->ctx, r, c));
        *o++ = '\n';
    }
    w->len = (size_t)(o - w->buf);
    return NULL;
}

int hio_write_text(FILE *fp, int rows, int cols, hio_value_fn f, const void *ctx)
{
    if (rows <= 0)
        return 0;
    int T = hio_threads();
    /* about 4 MB of text per task */
    int per = (int)((4u << 20) / ((size_t)cols * 18 + 1));
    if (per < 1)
        per = 1;
    if ((long long)T * per > rows)
        per = (rows + T - 1) / T;
    write_task *w = (write_task *)calloc((size_t)T, sizeof(write_task));
    if (!w)
        return 5;
    int rc = 0;
    for (int r = 0; r < rows && !rc; r += T * per) {
        int nt = 0;
        for (int t = 0; t < T; ++t) {
            int a = r + t * per, b = a + per;
            if (a >= rows)
                break;
            if (b > rows)
                b = rows;
            w[t].f = f;
            w[t].ctx = ctx;
            w[t].r0 = a;
            w[t].r1 = b;
            w[t].cols = cols;
            ++nt;
        }
        run_parallel(nt, format_rows, w, sizeof(write_task));
        for (int t = 0; t < nt && !rc; ++t) {
            if (w[t].oom)
                rc = 5;
            else if (fwrite(w[t].buf, 1, w[t].len, fp) != w[t].len)
                rc = 4;
        }
    }
    for (int t = 0; t < T; ++t)
        free(w[t].buf);
    free(w);
    return rc;
}

/* ---- binary format ------------------------------------------------------ */

static const char HIO_MAGIC[8] = {'H', 'C', 'F', 'B', 'I', 'N', '0', '1'};

static int little_endian(void)
{
    const uint32_t one = 1;
    unsigned char b;
    memcpy(&b, &one, 1);
    return b == 1;
}

static void put_i32(unsigned char *p, int v)
{
    uint32_t u = (uint32_t)v;
    p[0] = (unsigned char)(u & 255u);
    p[1] = (unsigned char)((u >> 8) & 255u);
    p[2] = (unsigned char)((u >> 16) & 255u);
    p[3] = (unsigned char)((u >> 24) & 255u);
}

static int get_i32(const unsigned char *p)
{
    return (int)((uint32_t)p[0] | ((uint32_t)p[1] << 8) | ((uint32_t)p[2] << 16) | ((uint32_t)p[3] << 24));
}

FILE *hio_bin_create(const char *path, int ndim, int n_x, int n_y, int nsnap, const double *times)
{
    if (!little_endian())  /* the planes are stored little-endian, as the host holds them */
        return NULL;
    FILE *fp = fopen(path, "wb");
    if (!fp)
        return NULL;
    unsigned char h[28];
    memcpy(h, HIO_MAGIC, 8);
    put_i32(h + 8, ndim);
    put_i32(h + 12, n_x);
    put_i32(h + 16, n_y);
    put_i32(h + 20, nsnap);
    put_i32(h + 24, 0);
    if (fwrite(h, 1, sizeof(h), fp) != sizeof(h) ||
        fwrite(times, sizeof(double), (size_t)nsnap, fp) != (size_t)nsnap) {
        fclose(fp);
        return NULL;
    }
    return fp;
}

int hio_bin_plane(FILE *fp, int rows, int cols, hio_value_fn f, const void *ctx)
{
    double *row = (double *)malloc(sizeof(double) * (size_t)(cols > 0 ? cols : 1));
    if (!row)
        return 5;
    int rc = 0;
    for (int r = 0; r < rows && !rc; ++r) {
        for (int c = 0; c < cols; ++c)
            row[c] = f(ctx, r, c);
        if (fwrite(row, sizeof(double), (size_t)cols, fp) != (size_t)cols)
            rc = 4;
    }
    free(row);
    return rc;
}

int hio_bin_read(const char *path, int *ndim, int *n_x, int *n_y, int *nsnap, double **times, double **data)
{
    *times = NULL;
    *data = NULL;
    if (!little_endian())
        return 4;
    FILE *fp = fopen(path, "rb");
    if (!fp)
        return 4;
    unsigned char h[28];
    if (fread(h, 1, sizeof(h), fp) != sizeof(h) || memcmp(h, HIO_MAGIC, 8) != 0) {
        fclose(fp);
        return 4;
    }
    *ndim = get_i32(h + 8);
    *n_x = get_i32(h + 12);
    *n_y = get_i32(h + 16);
    *nsnap = get_i32(h + 20);
    if (*ndim < 1 || *ndim > 2 || *n_x < 1 || *n_y < 1 || *nsnap < 1) {
        fclose(fp);
        return 4;
    }
    const size_t plane = (size_t)*n_x * (size_t)*n_y, total = plane * (size_t)*nsnap;
    *times = (double *)malloc(sizeof(double) * (size_t)*nsnap);
    *data = (double *)malloc(sizeof(double) * total);
    if (!*times || !*data) {
        free(*times);
        free(*data);
        *times = *data = NULL;
        fclose(fp);
        return 5;
    }
    int rc = 0;
    if (fread(*times, sizeof(double), (size_t)*nsnap, fp) != (size_t)*nsnap ||
        fread(*data, sizeof(double), total, fp) != total)
        rc = 4;
    fclose(fp);
    if (rc) {
        free(*times);
        free(*data);
        *times = *data = NULL;
    }
    return rc;
}
