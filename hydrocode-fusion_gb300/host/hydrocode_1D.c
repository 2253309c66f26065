/*
 * hydrocode_1D.c -- 1D driver linked against libhydro_gb300.so.
 *
 *   hydrocode_1D.out <in_example> <out_name> <order[_scheme]> EUL|LAG [n=C ...]
 *
 * Same command line, input folder, configuration and set-up as the
 * reference's src/hydrocode_1D/hydrocode.c:150-439: order 1 Godunov with the
 * exact Riemann solver, order 2 GRP, on Eulerian (EUL) or Lagrangian (LAG,
 * moving nodes X[k]) coordinates.  Exit codes as in the reference.
 * NODATPLOT suppresses the .dat output.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "hydro_io.h"

double config[N_CONF];

int main(int argc, char *argv[])
{
    for (int k = 1; k < N_CONF; k++)
        config[k] = INFINITY;
    arg_preprocess(4, argc, argv, NULL);
    config[0] = 1.0;
    int N, N_plot;
    double *time_plot;
    struct flu_var FV0 = initialize_1D(argv[1], &N, &N_plot, &time_plot);
    const int m = (int)config[3];
    const double h = config[10], gamma = config[6];
    const int order = (int)config[9];

    struct cell_var_stru CV;
    memset(&CV, 0, sizeof(CV));
    double *cpu_time = (double *)calloc(N, sizeof(double));
    double **X = (double **)malloc(N * sizeof(double *));
    CV.RHO = (double **)malloc(N * sizeof(double *));
    CV.U = (double **)malloc(N * sizeof(double *));
    CV.P = (double **)malloc(N * sizeof(double *));
    CV.E = (double **)malloc(N * sizeof(double *));
    if (!cpu_time || !X || !CV.RHO || !CV.U || !CV.P || !CV.E) {
        printf("NOT enough memory!\n");
        return 5;
    }
    CV.RHO[0] = FV0.RHO;
    CV.U[0] = FV0.U;
    CV.P[0] = FV0.P;
    for (int k = 0; k < N; ++k) {
        X[k] = (double *)malloc((m + 1) * sizeof(double));
        CV.E[k] = (double *)malloc(m * sizeof(double));
        if (k) {
            CV.RHO[k] = (double *)malloc(m * sizeof(double));
            CV.U[k] = (double *)malloc(m * sizeof(double));
            CV.P[k] = (double *)malloc(m * sizeof(double));
        }
        if (!X[k] || !CV.E[k] || !CV.RHO[k] || !CV.U[k] || !CV.P[k]) {
            printf("NOT enough memory! [%d]\n", k);
            return 5;
        }
    }
    for (int j = 0; j <= m; ++j)
        X[0][j] = h * j;
    for (int j = 0; j < m; ++j)
        CV.E[0][j] = 0.5 * CV.U[0][j] * CV.U[0][j] + CV.P[0][j] / (gamma - 1.0) / CV.RHO[0][j];
    if (strcmp(argv[4], "LAG") == 0) { /* hydrocode.c:237-251 */
        config[8] = 1.0;
        switch (order) {
        case 1:
            Godunov_solver_LAG_source(m, CV, X, cpu_time, &N, time_plot);
            break;
        case 2:
            GRP_solver_LAG_source(m, CV, X, cpu_time, &N, time_plot);
            break;
        default:
            printf("NOT appropriate order of the scheme! The order is %d.\n", order);
            return 4;
        }
    } else if (strcmp(argv[4], "EUL") == 0) { /* hydrocode.c:252-270 */
        config[8] = 0.0;
        for (int k = 1; k < N; ++k)
            for (int j = 0; j <= m; ++j)
                X[k][j] = X[0][j];
        switch (order) {
        case 1:
            Godunov_solver_EUL_source(m, CV, cpu_time, &N, time_plot);
            break;
        case 2:
            GRP_solver_EUL_source(m, CV, cpu_time, &N, time_plot);
            break;
        default:
            printf("NOT appropriate order of the scheme! The order is %d.\n", order);
            return 4;
        }
    } else {
        printf("NOT appropriate coordinate framework! The framework is %s.\n", argv[4]);
        return 4;
    }
#ifndef NODATPLOT
    file_1D_write(m, N, CV, X, cpu_time, argv[2], time_plot);
#endif
    return 0;
}
