/*
 * hydro_io.h -- C99 host side of the drop-in: the data_in readers, the
 * data_out writers, configuration handling and the command-line conventions
 * of HydroCODE's 1D/2D drivers, restated for the GB300 library.
 *
 * Formats and conventions follow the reference's src/file_io/ (file:line in
 * each function's comment): config files of "index value" lines ('#' starts a
 * comment, a value given on the command line as "n=C" wins), whitespace
 * separated initial data RHO/U/(V)/P.txt|.dat (2D files: one line per y row),
 * an optional time_plot.txt|.dat, and %.10g text output under
 * ../../data_out/<dim>/<EUL_|LAG_|ALE_><order>_order/<name>/ (relative to the
 * driver's working directory, as in the reference; HYDRO_DATA_ROOT overrides
 * the "../../" prefix).
 * Beyond the reference: the data files are read and the text written by
 * several threads (hydro_fastio.h; the same numbers and bytes), an initial
 * data file may also be <var>.bin (the binary FP64 format, used when no .txt
 * or .dat exists), and config[302] = 1 adds binary output <var>.bin beside
 * the .dat files, 2 writes only the binary files.
 */
#ifndef HYDRO_IO_H
#define HYDRO_IO_H

#include <stdio.h>

#include "../../include/hydro_gb300.h"

/* Pointers to one initial data set (the reference's struct flu_var, single fluid). */
struct flu_var {
    double *RHO, *U, *V, *P;
};

void example_io(const char *example, char *add_mkdir, const int i_or_o);
int CreateDir(const char *pPath);
int flu_var_count(FILE *fp, const char *add);
int flu_var_count_line(FILE *fp, const char *add, int *n_x);
int flu_var_read(FILE *fp, double *U, const int num);
int time_plot_read(const char *add_in, const int N_max, int *N_plot, double *time_plot[]);
void arg_preprocess(const int argc_least, const int argc, char *argv[], char *scheme);
void configurate(const char *add_in);
void config_write(const char *add_out, const double *cpu_time, const char *name);
struct flu_var initialize_1D(const char *name, int *N, int *N_plot, double *time_plot[]);
struct flu_var initialize_2D(const char *name, int *N, int *N_plot, double *time_plot[]);
void file_1D_write(const int m, const int N, const struct cell_var_stru CV, double *X[], const double *cpu_time,
                   const char *problem, const double time_plot[]);
void file_2D_write(const int n_x, const int n_y, const int N, const struct cell_var_stru CV[], double **X, double **Y,
                   const double *cpu_time, const char *problem, const double time_plot[]);
void file_2D_write_POINT_TEC(const int n_x, const int n_y, const int N, const struct cell_var_stru CV[], double **X,
                             double **Y, const double *cpu_time, const char *problem, const double time_plot[]);

#endif
