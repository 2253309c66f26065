/*
 * hydrocode_2D.c -- 2D Eulerian driver linked against libhydro_gb300.so.
 *
 *   hydrocode_2D.out <in_example> <out_name> <order[_scheme]> EUL [n=C ...]
 *
 * Same command line, input folder, configuration, allocation of the x-major
 * cell arrays and energy initialisation as the reference's
 * src/hydrocode_2D/hydrocode.c:164-470; the scheme call is the library's.
 * Exit codes: 0 fine, 1 file error, 2 data error, 4 argument error, 5 memory.
 * Compile-time switches as in the reference: NODATPLOT (no .dat output),
 * NOTECPLOT (no Tecplot output).  config[300] selects the GPU form.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "hydro_io.h"

double config[N_CONF];

static double **alloc_rows(int a, int b)
{
    double **p = (double **)malloc(a * sizeof(double *));
    if (!p)
        return NULL;
    for (int j = 0; j < a; ++j)
        if (!(p[j] = (double *)malloc(b * sizeof(double))))
            return NULL;
    return p;
}

int main(int argc, char *argv[])
{
    for (int k = 1; k < N_CONF; k++)
        config[k] = INFINITY;
    arg_preprocess(4, argc, argv, NULL);
    config[0] = 2.0;
    int N, N_plot;
    double *time_plot;
    struct flu_var FV0 = initialize_2D(argv[1], &N, &N_plot, &time_plot);
    const int n_x = (int)config[13], n_y = (int)config[14];
    const double h_x = config[10], h_y = config[11], gamma = config[6];
    const int order = (int)config[9];
    const int dim_split = (int)config[33];

    struct cell_var_stru *CV = (struct cell_var_stru *)calloc(N, sizeof(struct cell_var_stru));
    double *cpu_time = (double *)calloc(N, sizeof(double));
    double **X = alloc_rows(n_x + 1, n_y + 1), **Y = alloc_rows(n_x + 1, n_y + 1);
    if (!CV || !cpu_time || !X || !Y) {
        printf("NOT enough memory! Cell Variables\n");
        return 5;
    }
    for (int k = 0; k < N; ++k) {
        CV[k].RHO = alloc_rows(n_x, n_y);
        CV[k].U = alloc_rows(n_x, n_y);
        CV[k].V = alloc_rows(n_x, n_y);
        CV[k].P = alloc_rows(n_x, n_y);
        CV[k].E = alloc_rows(n_x, n_y);
        if (!CV[k].RHO || !CV[k].U || !CV[k].V || !CV[k].P || !CV[k].E) {
            printf("NOT enough memory! CV[%d]\n", k);
            return 5;
        }
    }
    for (int j = 0; j <= n_x; ++j)
        for (int i = 0; i <= n_y; ++i) {
            X[j][i] = j * h_x;
            Y[j][i] = i * h_y;
        }
    /* file row i is y index i: transpose into the x-major arrays */
    for (int j = 0; j < n_x; ++j)
        for (int i = 0; i < n_y; ++i) {
            CV[0].RHO[j][i] = FV0.RHO[i * n_x + j];
            CV[0].U[j][i] = FV0.U[i * n_x + j];
            CV[0].V[j][i] = FV0.V[i * n_x + j];
            CV[0].P[j][i] = FV0.P[i * n_x + j];
            CV[0].E[j][i] = 0.5 * CV[0].U[j][i] * CV[0].U[j][i] + CV[0].P[j][i] / (gamma - 1.0) / CV[0].RHO[j][i];
            CV[0].E[j][i] += 0.5 * CV[0].V[j][i] * CV[0].V[j][i];
        }
    if (strcmp(argv[4], "EUL") != 0) {
        printf("NOT appropriate coordinate framework! The framework is %s.\n", argv[4]);
        return 4;
    }
    config[8] = 0.0;
    switch (order) {
    case 1:
        config[41] = 0.0; /* alpha = 0: first order from the second-order scheme */
        /* fall through */
    case 2:
        if (dim_split)
            GRP_solver_2D_split_EUL_source(n_x, n_y, CV, X, Y, cpu_time, argv[2], N, &N_plot, time_plot);
        else
            GRP_solver_2D_EUL_source(n_x, n_y, CV, X, Y, cpu_time, argv[2], N, &N_plot, time_plot);
        break;
    default:
        printf("NOT appropriate order of the scheme! The order is %d.\n", order);
        return 4;
    }
#ifndef NODATPLOT
    file_2D_write(n_x, n_y, N_plot, CV, X, Y, cpu_time, argv[2], time_plot);
#endif
#ifndef NOTECPLOT
    /* stored plot snapshots, then the final state */
    for (int k = 0; k + 1 < N_plot; ++k)
        file_2D_write_POINT_TEC(n_x, n_y, 1, CV + k, X, Y, cpu_time, argv[2], time_plot + k);
    file_2D_write_POINT_TEC(n_x, n_y, 1, CV + N_plot - 1, X, Y, cpu_time, argv[2], time_plot + N_plot - 1);
#endif
    return 0;
}
