/*
 * hydro_io.c -- data_in readers, data_out writers and configuration handling
 * of the GB300 drivers (C99).  Same file formats, directory conventions,
 * defaults and error exits as the reference's src/file_io/.
 */
#include <ctype.h>
#include <errno.h>
#include <limits.h>
#include <math.h>
#include <stdbool.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/stat.h>
#include <sys/types.h>
#include <unistd.h>

#include "hydro_fastio.h"
#include "hydro_io.h"

#define PATH_LEN (FILENAME_MAX + 40)

static const char *data_root(void)
{
    const char *r = getenv("HYDRO_DATA_ROOT");
    return (r && *r) ? r : "../../";
}

/* mkdir -p; -1 if it already existed and is writable, 0 if created, 1 on failure
 * (src/tools/sys_pro.c:72). */
int CreateDir(const char *pPath)
{
    char tmp[PATH_LEN];
    size_t len = strlen(pPath);
    if (access(pPath, W_OK) == 0)
        return -1;
    if (len >= sizeof(tmp))
        return 1;
    memcpy(tmp, pPath, len + 1);
    for (size_t k = 1; k <= len; ++k)
        if (tmp[k] == '/' || tmp[k] == '\0') {
            char c = tmp[k];
            tmp[k] = '\0';
            if (access(tmp, F_OK) != 0)
                mkdir(tmp, 0777);
            tmp[k] = c;
        }
    return access(pPath, W_OK) == 0 ? 0 : 1;
}

/* Input folder <root>data_in/<dim>/<example>/ or output folder
 * <root>data_out/<dim>/<EUL_|LAG_|ALE_><order>_order/<example>/
 * (src/file_io/io_control.c:40-115). */
void example_io(const char *example, char *add_mkdir, const int i_or_o)
{
    const int dim = (int)config[0], el = (int)config[8], order = (int)config[9];
    static int announced = 0;
    const char *sdim = dim == 1 ? "one-dim/" : dim == 2 ? "two-dim/" : dim == 3 ? "three-dim/" : NULL;
    if (!sdim) {
        fprintf(stderr, "Strange computational dimension!\n");
        exit(2);
    }
    if (i_or_o == 0) {
        const char *sel = el == 0 ? "EUL_" : el == 1 ? "LAG_" : el == 2 ? "ALE_" : NULL;
        if (!sel) {
            fprintf(stderr, "Strange description method of fluid motion!\n");
            exit(2);
        }
        snprintf(add_mkdir, PATH_LEN, "%sdata_out/%s%s%d_order/%s", data_root(), sdim, sel, order, example);
        if (CreateDir(add_mkdir) == 1) {
            fprintf(stderr, "Output directory '%s' construction failed!\n", add_mkdir);
            exit(1);
        } else if (!announced) {
            printf("Output directory '%s' has been constructed.\n", add_mkdir);
            announced = 1;
        }
    } else {
        snprintf(add_mkdir, PATH_LEN, "%sdata_in/%s%s", data_root(), sdim, example);
        if (access(add_mkdir, R_OK) == -1) {
            fprintf(stderr, "Input directory '%s' is nonexistent or unreadable!\n", add_mkdir);
            exit(1);
        }
    }
    strcat(add_mkdir, "/");
}

static int number_char(int ch) { return ch == '-' || ch == '.' || ch == 'E' || ch == 'e' || isdigit(ch); }

/* Count of numbers in a whitespace-separated file (io_control.c:124-161). */
int flu_var_count(FILE *fp, const char *add)
{
    int num = 0, flg = 0, ch;
    while ((ch = getc(fp)) != EOF) {
        if (number_char(ch))
            flg = 1;
        else if (!isspace(ch)) {
            fprintf(stderr, "Input contains illegal character(ASCII=%d, flag=%d) in the file '%s'!\n", ch, flg, add);
            return 0;
        } else if (flg) {
            num++;
            flg = 0;
        }
    }
    rewind(fp);
    return num;
}

/* Lines of numbers and the common column count (io_control.c:163-215). */
int flu_var_count_line(FILE *fp, const char *add, int *n_x)
{
    int line = 0, column = 0, flag = 0, ch;
    do {
        ch = getc(fp);
        if (ch == '\n' || ch == EOF) {
            if (flag)
                ++column;
            flag = 0;
            if (column) {
                if (!line)
                    *n_x = column;
                else if (column != *n_x) {
                    printf("Error in input data file '%s', line=%d, column=%d, n_x=%d\n", add, line, column, *n_x);
                    return 0;
                }
                ++line;
                column = 0;
            }
        } else if (number_char(ch))
            flag = 1;
        else if (!isspace(ch)) {
            printf("Input contains illigal character(ASCII=%d, flag=%d) in the file '%s', line=%d!\n", ch, flag, add, line);
            return 0;
        } else if (flag) {
            ++column;
            flag = 0;
        }
    } while (ch != EOF);
    rewind(fp);
    return line;
}

/* Reads num numbers with strtod; returns 0 or the index of the bad entry
 * (io_control.c:221-261). */
int flu_var_read(FILE *fp, double *U, const int num)
{
    int idx = 0, j = 0, ch;
    char number[100], *endptr;
    while ((ch = getc(fp)) != EOF) {
        if (isspace(ch) && idx) {
            number[idx] = '\0';
            idx = 0;
            errno = 0;
            double v = strtod(number, &endptr);
            if (errno == ERANGE || *endptr != '\0') {
                printf("The %dth entry in the initial data file is not a double-precision floats.\n", j + 1);
                return j + 1;
            } else if (j == num) {
                printf("Error on the initial data file reading!\n");
                return j;
            }
            U[j++] = v;
        } else if (number_char(ch) && idx < 99)
            number[idx++] = (char)ch;
    }
    return 0;
}

static int compare_double(const void *a, const void *b)
{
    double r = *(const double *)a - *(const double *)b;
    return r > 0.0 ? 1 : (r < 0.0 ? -1 : 0);
}

/* time_plot.txt|.dat: plot times; N_plot = count + 2, time_plot[0] = 0,
 * time_plot[N_plot-1] = config[1]; returns min(N_max, N_plot)
 * (io_control.c:288-335). */
int time_plot_read(const char *add_in, const int N_max, int *N_plot, double *time_plot[])
{
    char add[PATH_LEN];
    FILE *fp;
    bool r = true;
    snprintf(add, sizeof(add), "%stime_plot.txt", add_in);
    if ((fp = fopen(add, "r")) == NULL) {
        snprintf(add, sizeof(add), "%stime_plot.dat", add_in);
        fp = fopen(add, "r");
    }
    if (fp == NULL) {
        printf("No time data file for plotting! Only the initial data and final result will be plotted.\n");
        *N_plot = 2;
        r = false;
    } else
        *N_plot = flu_var_count(fp, add) + 2;
    if (*N_plot < 2) {
        printf("Error in counting time data file for plotting!\n");
        exit(2);
    }
    *time_plot = (double *)malloc((*N_plot) * sizeof(double));
    if (*time_plot == NULL) {
        printf("NOT enough memory! time_plot[]\n");
        exit(5);
    }
    (*time_plot)[0] = 0.0;
    (*time_plot)[*N_plot - 1] = config[1];
    if (r) {
        if (flu_var_read(fp, *time_plot + 1, *N_plot - 2)) {
            fclose(fp);
            exit(2);
        }
        printf("Load time data file for plotting! Plot time step is %d.\n", *N_plot - 2);
        qsort(*time_plot, *N_plot - 1, sizeof(double), compare_double);
        fclose(fp);
    }
    return N_max < (*N_plot) ? N_max : (*N_plot);
}

/* argv[3] = order[_scheme] -> config[9]; "n=C" arguments -> config[n]
 * (src/file_io/terminal_io.c:26-105). */
void arg_preprocess(const int argc_least, const int argc, char *argv[], char *scheme)
{
    (void)scheme;
    printf("\n");
    for (int k = 0; k < argc; k++)
        printf("%s ", argv[k]);
    printf("\n\n");
    if (argc < argc_least) {
        printf("Test Beginning: ARGuments Counter %d is less than %d\n", argc, argc_least);
        exit(4);
    }
    printf("TEST:\n %s\n", argv[1]);
    char *endp;
    errno = 0;
    unsigned long order = strtoul(argv[3], &endp, 10);
    if (*endp == '_')
        endp++;
    else if (*endp != '\0' || errno == ERANGE) {
        printf("No order or Wrog scheme!\n");
        exit(4);
    }
    config[9] = (double)order;
    for (int k = argc_least + 1; k < argc; k++) {
        errno = 0;
        unsigned long j = strtoul(argv[k], &endp, 10);
        if (errno != ERANGE && *endp == '=' && j < N_CONF) {
            endp++;
            errno = 0;
            double v = strtod(endp, &endp);
            if (errno != ERANGE && *endp == '\0') {
                config[j] = v;
                printf("%3lu-th configuration: %g (ARGument)\n", j, v);
            } else {
                printf("Configuration error in ARGument variable %d! ERROR after '='!\n", k);
                exit(4);
            }
        } else {
            printf("Configuration error in ARGument variable %d! ERROR before '='!\n", k);
            exit(4);
        }
    }
}

/* Defaults and range checks (src/file_io/config_handle.c:39-152). */
static void config_check(void)
{
    const int dim = (int)config[0];
    if (isfinite(config[1]) && config[1] >= 0.0)
        config[5] = isfinite(config[5]) ? config[5] : (double)INT_MAX;
    else if (!isfinite(config[5])) {
        fprintf(stderr, "The total time or the maximum number of time steps must be setted properly!\n");
        exit(2);
    } else
        config[1] = INFINITY;
    if (isinf(config[4]))
        config[4] = 1e-9;
    if (config[4] < 0.0 || config[4] > 0.01) {
        fprintf(stderr, "eps(%f) should in (0, 0.01)!\n", config[4]);
        exit(2);
    }
    if (isinf(config[6]))
        config[6] = 1.4;
    else if (config[6] < 1.0 + config[4]) {
        fprintf(stderr, "The constant of the perfect gas(%f) should be larger than 1.0!\n", config[6]);
        exit(2);
    }
    if (isinf(config[7]))
        config[7] = dim == 1 ? 0.9 : 0.45;
    else if (config[7] > 1.0 - config[4]) {
        fprintf(stderr, "The CFL number(%f) should be smaller than 1.0.\n", config[7]);
        exit(2);
    }
    if (isinf(config[41]))
        config[41] = 1.9;
    else if (config[41] < -config[4] || config[41] > 2.0) {
        fprintf(stderr, "The parameter in minmod limiter(%f) should in [0, 2)!\n", config[41]);
        exit(2);
    }
    if (isinf(config[110]))
        config[110] = 0.72;
    config[2] = isfinite(config[2]) ? config[2] : 1.0;
    config[8] = isfinite(config[8]) ? config[8] : 0.0;
    config[20] = isfinite(config[20]) ? config[20] : config[10];
    config[30] = isfinite(config[30]) ? config[30] : 0.0;
    config[31] = isfinite(config[31]) ? config[31] : 0.0;
    config[32] = isfinite(config[32]) ? config[32] : 1.0;
    config[33] = isfinite(config[33]) ? config[33] : 0.0;
    config[40] = isfinite(config[40]) ? config[40] : 0.0;
    config[42] = isfinite(config[42]) ? config[42] : 1.0;
    config[53] = isfinite(config[53]) ? config[53] : 0.0;
    config[60] = isfinite(config[60]) ? config[60] : 0.0;
    config[61] = isfinite(config[61]) ? config[61] : 0.0;
    config[70] = isfinite(config[70]) ? config[70] : 0.0;
    config[210] = isfinite(config[210]) ? config[210] : 0.0;
    config[211] = isfinite(config[211]) ? config[211] : 0.0;
    config[212] = isfinite(config[212]) ? config[212] : 0.0;
}

/* "index value" lines; a value already set (command line) is kept
 * (config_handle.c:162-200). */
static int config_read(FILE *fp)
{
    char line[200], *endp;
    int line_num = 1;
    while (fgets(line, sizeof(line), fp) != NULL) {
        long i = strtol(line, &endp, 10);
        while (isspace((unsigned char)*endp))
            endp++;
        if (0 < i && i < N_CONF) {
            errno = 0;
            double v = strtod(endp, NULL);
            if (errno == ERANGE) {
                fprintf(stderr, "Value range error of %ld-th configuration in line %d of configuration file!\n", i,
                        line_num);
                return 1;
            } else if (isinf(config[i]))
                printf("%3ld-th configuration: %g\n", i, config[i] = v);
            else if (fabs(config[i] - v) > 1e-9)
                printf("%3ld-th configuration is repeatedly assigned with %g and %g(abandon)!\n", i, config[i], v);
        } else if (i != 0 || (*endp != '#' && *endp != '\0'))
            fprintf(stderr, "Warning: unknown row occurrs in line %d of configuration file!\n", line_num);
        line_num++;
    }
    return ferror(fp) ? 0 : 1;
}

void configurate(const char *add_in)
{
    char add[PATH_LEN];
    FILE *fp;
    snprintf(add, sizeof(add), "%sconfig.txt", add_in);
    if ((fp = fopen(add, "r")) == NULL) {
        snprintf(add, sizeof(add), "%sconfig.dat", add_in);
        fp = fopen(add, "r");
    }
    if (fp == NULL) {
        printf("Cannot open configuration data file!\n");
        perror(add_in);
        exit(1);
    }
    if (config_read(fp) == 0) {
        fclose(fp);
        exit(2);
    }
    fclose(fp);
    printf("Configurated:\n");
    config_check();
}

/* log.dat (config_handle.c:253-303). */
void config_write(const char *add_out, const double *cpu_time, const char *name)
{
    (void)cpu_time;
    char file[PATH_LEN];
    const int dim = (int)config[0];
    snprintf(file, sizeof(file), "%slog.dat", add_out);
    FILE *fp = fopen(file, "w");
    if (!fp) {
        printf("Cannot open log output file!\n");
        exit(1);
    }
    fprintf(fp, "%s is initialized with %d grids.\n\n", name, (int)config[3]);
    fprintf(fp, "Configurated:\n");
    fprintf(fp, "dim\t\t= %d\n", dim);
    if (isfinite(config[1]))
        fprintf(fp, "t_all\t= %d\n", (int)config[1]);
    else if (isfinite(config[16]))
        fprintf(fp, "tau\t\t= %g\n", config[16]);
    fprintf(fp, "eps\t\t= %g\n", config[4]);
    fprintf(fp, "gamma\t= %g\n", config[6]);
    fprintf(fp, "CFL\t\t= %g\n", config[7]);
    fprintf(fp, "h\t\t= %g\n", config[10]);
    fprintf(fp, "bond\t= %d\n", (int)config[17]);
    if (dim == 2) {
        fprintf(fp, "h_y\t\t= %g\n", config[11]);
        fprintf(fp, "bond_y\t= %d\n", (int)config[18]);
    }
    fprintf(fp, "\nA total of %d time steps are computed.\n", (int)config[5]);
    fclose(fp);
}

/* Initial data file of one variable: <var>.txt, else <var>.dat (as the
 * reference, file_1D_in.c:104-110), else <var>.bin (the binary FP64 format of
 * hydro_fastio.h).  Returns 1 text, 2 binary, 0 none (after the reference's
 * message). */
static int find_input(const char *add_in, const char *var, char *add)
{
    static const char *ext[3] = {"txt", "dat", "bin"};
    for (int e = 0; e < 3; ++e) {
        snprintf(add, PATH_LEN, "%s%s.%s", add_in, var, ext[e]);
        if (access(add, R_OK) == 0)
            return e < 2 ? 1 : 2;
    }
    printf("Cannot open initial data file: %s!\n", var);
    return 0;
}

/* Numbers of one initial data file: *lines x *columns (2D text: lines are y
 * rows; binary: n_y x n_x of its first plane).  Exits as the reference's
 * initialisation does on a read error (2 data, 5 memory). */
static double *read_input(const char *add, int kind, int check_columns, int *lines, int *columns, long long *num)
{
    double *d = NULL;
    if (kind == 2) {
        int ndim, n_x, n_y, nsnap;
        double *times = NULL;
        int rc = hio_bin_read(add, &ndim, &n_x, &n_y, &nsnap, &times, &d);
        free(times);
        if (rc) {
            printf("Error in reading the binary initial data file '%s'!\n", add);
            exit(rc == 5 ? 5 : 2);
        }
        *lines = n_y;
        *columns = n_x;
        *num = (long long)n_x * n_y;  /* the first plane */
        return d;
    }
    int rc = hio_read_table(add, check_columns, lines, columns, num, &d);
    if (rc == 5) {
        printf("NOT enough memory! %s\n", add);
        exit(5);
    }
    if (rc == 3)  /* an entry strtod does not take: the reference's flu_var_read failure */
        exit(2);
    if (rc || *num < 1) {
        printf("Error in counting fluid variables in initial data file: %s!\n", add);
        exit(2);
    }
    return d;
}

/* 1D initial data (src/file_io/file_1D_in.c:93-151); the numbers are read by
 * hio_read_table (several threads, the same values as the reference's getc
 * reader). */
struct flu_var initialize_1D(const char *name, int *N, int *N_plot, double *time_plot[])
{
    struct flu_var FV0 = {NULL, NULL, NULL, NULL};
    char add_in[PATH_LEN], add[PATH_LEN];
    example_io(name, add_in, 1);
    configurate(add_in);
    *N = time_plot_read(add_in, 1000, N_plot, time_plot);
    const char *vars[3] = {"RHO", "U", "P"};
    double **dst[3] = {&FV0.RHO, &FV0.U, &FV0.P};
    for (int q = 0; q < 3; ++q) {
        int kind = find_input(add_in, vars[q], add);
        if (!kind)
            exit(1);
        int lines, columns;
        long long num;
        *dst[q] = read_input(add, kind, 0, &lines, &columns, &num);
        if (isinf(config[3]))
            config[3] = (double)num;
        else if (num != (long long)config[3]) {
            printf("Input unequal! num_%s=%lld, num_cell=%d.\n", vars[q], num, (int)config[3]);
            exit(2);
        }
    }
    printf("'%s' data initialized, grid cell number = %d.\n", add_in, (int)config[3]);
    return FV0;
}

/* 2D initial data: line x column numbers per file, rows are y
 * (src/file_io/file_2D_in.c:28-67, 119-179). */
struct flu_var initialize_2D(const char *name, int *N, int *N_plot, double *time_plot[])
{
    struct flu_var FV0 = {NULL, NULL, NULL, NULL};
    char add_in[PATH_LEN], add[PATH_LEN];
    example_io(name, add_in, 1);
    configurate(add_in);
    *N = time_plot_read(add_in, 5, N_plot, time_plot);
    const char *vars[4] = {"RHO", "U", "V", "P"};
    double **dst[4] = {&FV0.RHO, &FV0.U, &FV0.V, &FV0.P};
    for (int q = 0; q < 4; ++q) {
        int kind = find_input(add_in, vars[q], add);
        if (!kind)
            exit(1);
        int line, column;
        long long num;
        *dst[q] = read_input(add, kind, 1, &line, &column, &num);
        if (isinf(config[3]))
            config[3] = (double)num;
        if (isinf(config[13]))
            config[13] = (double)column;
        if (isinf(config[14]))
            config[14] = (double)line;
        else if (num != (long long)config[3] || column != (int)config[13] || line != (int)config[14]) {
            printf("Input unequal! %s\n", add);
            exit(2);
        }
    }
    printf("'%s' data initialized, line = %d, column = %d.\n", add_in, (int)config[14], (int)config[13]);
    return FV0;
}

static FILE *open_output(const char *add_out, const char *var)
{
    char file[PATH_LEN];
    snprintf(file, sizeof(file), "%s%s.dat", add_out, var);
    FILE *fp = fopen(file, "w");
    if (!fp) {
        printf("Cannot open solution output file: %s!\n", var);
        exit(1);
    }
    return fp;
}

static void write_time_plot(const char *add_out, const int N, const double time_plot[])
{
    FILE *fp = open_output(add_out, "time_plot");
    for (int k = 0; k < N; ++k)
        fprintf(fp, "%.10g\n", time_plot[k]);
    fclose(fp);
}

/* Output formats, config[302] (unused by the reference): 0 or absent = the
 * reference's %.10g text, 1 = text and binary (<var>.bin, hydro_fastio.h),
 * 2 = binary only. */
static int out_text(void) { return !(isfinite(config[302]) && (int)config[302] == 2); }
static int out_bin(void) { return isfinite(config[302]) && ((int)config[302] == 1 || (int)config[302] == 2); }

/* value accessors of the writers: one row of a plane per call site */
typedef struct {
    double **a;       /* 2D: a[j][i] = x-major cell array; 1D: a[k][j] */
    double **X, **Y;  /* 2D node coordinates */
    int q, k;
} out_ctx;

static double val_1d(const void *ctx, int r, int c)
{
    const out_ctx *o = (const out_ctx *)ctx;
    return o->a[o->k + r][c];
}
static double val_1d_x(const void *ctx, int r, int c)
{
    const out_ctx *o = (const out_ctx *)ctx;
    return 0.5 * (o->X[o->k + r][c] + o->X[o->k + r][c + 1]);
}
static double val_2d(const void *ctx, int r, int c)
{
    const out_ctx *o = (const out_ctx *)ctx;
    return o->a[c][r];  /* row r = y index i, column c = x index j */
}
static double val_2d_center(const void *ctx, int r, int c)
{
    const out_ctx *o = (const out_ctx *)ctx;
    double **Z = o->q == 5 ? o->X : o->Y;
    return 0.25 * (Z[c][r] + Z[c][r + 1] + Z[c + 1][r] + Z[c + 1][r + 1]);
}

/* 1D binary output: N snapshots of one row of m values. */
static void write_bin_1d(const char *add_out, const char *var, int m, int N, const double time_plot[], out_ctx *o,
                         hio_value_fn f)
{
    char file[PATH_LEN + 64];
    snprintf(file, sizeof(file), "%s%s.bin", add_out, var);
    FILE *fp = hio_bin_create(file, 1, m, 1, N, time_plot);
    if (!fp) {
        printf("Cannot open solution output file: %s!\n", var);
        exit(1);
    }
    int rc = 0;
    for (int k = 0; k < N && !rc; ++k) {
        o->k = k;
        rc = hio_bin_plane(fp, 1, m, f, o);
    }
    if (fclose(fp) != 0 || rc) {
        printf("Error in writing solution output file: %s!\n", var);
        exit(1);
    }
}

/* 1D .dat output: one line per stored time (src/file_io/file_1D_out.c:49-95);
 * the lines are formatted by several threads (the same bytes). */
void file_1D_write(const int m, const int N, const struct cell_var_stru CV, double *X[], const double *cpu_time,
                   const char *problem, const double time_plot[])
{
    char add_out[PATH_LEN];
    example_io(problem, add_out, 0);
    double **vars[4] = {CV.RHO, CV.U, CV.P, CV.E};
    const char *names[5] = {"RHO", "U", "P", "E", "X"};
    for (int q = 0; q < 5; ++q) {
        out_ctx o = {q < 4 ? vars[q] : NULL, X, NULL, q, 0};
        hio_value_fn f = q < 4 ? val_1d : val_1d_x;
        if (out_text()) {
            FILE *fp = open_output(add_out, names[q]);
            if (hio_write_text(fp, N, m, f, &o)) {
                printf("Error in writing solution output file: %s!\n", names[q]);
                exit(1);
            }
            fclose(fp);
        }
        if (out_bin())
            write_bin_1d(add_out, names[q], m, N, time_plot, &o, f);
    }
    write_time_plot(add_out, N, time_plot);
    config_write(add_out, cpu_time, problem);
}

/* 2D .dat output: per stored time, one line per y row, blank lines between
 * times (src/file_io/file_2D_out.c:55-101); rows formatted by several threads
 * (the same bytes). */
void file_2D_write(const int n_x, const int n_y, const int N, const struct cell_var_stru CV[], double **X, double **Y,
                   const double *cpu_time, const char *problem, const double time_plot[])
{
    char add_out[PATH_LEN];
    example_io(problem, add_out, 0);
    const char *names[7] = {"RHO", "U", "V", "P", "E", "X", "Y"};
    for (int q = 0; q < 7; ++q) {
        out_ctx o = {NULL, X, Y, q, 0};
        hio_value_fn f = q < 5 ? val_2d : val_2d_center;
        FILE *fp = out_text() ? open_output(add_out, names[q]) : NULL;
        FILE *bp = NULL;
        if (out_bin()) {
            char file[PATH_LEN + 64];
            snprintf(file, sizeof(file), "%s%s.bin", add_out, names[q]);
            bp = hio_bin_create(file, 2, n_x, n_y, N, time_plot);
            if (!bp) {
                printf("Cannot open solution output file: %s!\n", names[q]);
                exit(1);
            }
        }
        for (int k = 0; k < N; ++k) {
            switch (q) {
            case 0: o.a = CV[k].RHO; break;
            case 1: o.a = CV[k].U; break;
            case 2: o.a = CV[k].V; break;
            case 3: o.a = CV[k].P; break;
            case 4: o.a = CV[k].E; break;
            default: break;
            }
            if (fp && (hio_write_text(fp, n_y, n_x, f, &o) || fprintf(fp, "\n\n") < 0)) {
                printf("Error in writing solution output file: %s!\n", names[q]);
                exit(1);
            }
            if (bp && hio_bin_plane(bp, n_y, n_x, f, &o)) {
                printf("Error in writing solution output file: %s!\n", names[q]);
                exit(1);
            }
        }
        if (fp)
            fclose(fp);
        if (bp && fclose(bp) != 0) {
            printf("Error in writing solution output file: %s!\n", names[q]);
            exit(1);
        }
    }
    write_time_plot(add_out, N, time_plot);
    config_write(add_out, cpu_time, problem);
}

/* Tecplot point data FLU_VAR_<t>.tec (src/file_io/file_2D_out.c:103-151). */
void file_2D_write_POINT_TEC(const int n_x, const int n_y, const int N, const struct cell_var_stru CV[], double **X,
                             double **Y, const double *cpu_time, const char *problem, const double time_plot[])
{
    (void)cpu_time;
    char add_out[PATH_LEN], file[PATH_LEN + 64];
    example_io(problem, add_out, 0);
    snprintf(file, sizeof(file), "%sFLU_VAR_%.8g.tec", add_out, time_plot[N - 1] + config[4]);
    FILE *fp = fopen(file, "w");
    if (!fp) {
        fprintf(stderr, "Cannot open solution output TECPLOT file of '%s'!\n", problem);
        exit(1);
    }
    fprintf(fp, "TITLE = \"FE-Volume Point Data\"\n");
    fprintf(fp, "VARIABLES = \"X\", \"Y\", \"P\", \"RHO\", \"U\", \"V\", \"E\"\n");
    for (int k = 0; k < N; ++k) {
        fprintf(fp, "ZONE I=%d, J=%d, SOLUTIONTIME=%.10g, DATAPACKING=POINT\n", n_x, n_y, time_plot[k]);
        for (int i = 0; i < n_y; ++i)
            for (int j = 0; j < n_x; ++j) {
                fprintf(fp, "%.10g\t", 0.25 * (X[j][i] + X[j][i + 1] + X[j + 1][i] + X[j + 1][i + 1]));
                fprintf(fp, "%.10g\t", 0.25 * (Y[j][i] + Y[j][i + 1] + Y[j + 1][i] + Y[j + 1][i + 1]));
                fprintf(fp, "%.10g\t%.10g\t%.10g\t%.10g\t%.10g\t\n", CV[k].P[j][i], CV[k].RHO[j][i], CV[k].U[j][i],
                        CV[k].V[j][i], CV[k].E[j][i]);
            }
        fprintf(fp, "\n");
    }
    fclose(fp);
}
