/*
 * Force-included ahead of the reference sources when they are compiled into
 * oracle/_ref.  It defines the reference's include guard SOLVELIN_H first, so
 * the reference's own n_solvelin.hpp (include/cpu/n_solvelin.hpp:13-50, whose
 * back-substitution starts at k = rows and reads/writes index 3 of 3-element
 * arrays) is skipped and this correct Gauss elimination is used instead.
 * Elimination follows the same no-pivot row order (:28-35); back-substitution
 * runs k = e-1 .. 0 over columns m > k.
 */
#ifndef SOLVELIN_H
#define SOLVELIN_H
#include <iostream>

template <class T>
void solvelin(T A[3][3], T b[3], T x[3], int e, int method)
{
    if (method != 1) return;
    for (int k = 0; k < e - 1; k++)
        for (int n = k; n < e - 1; n++) {
            T a = A[n + 1][k] / A[k][k];
            for (int m = 0; m < e; m++) A[n + 1][m] = A[n + 1][m] - a * A[k][m];
            b[n + 1] = b[n + 1] - a * b[k];
        }
    for (int k = e - 1; k >= 0; k--) {
        T c = b[k];
        for (int m = e - 1; m > k; m--) c = c - A[k][m] * x[m];
        x[k] = c / A[k][k];
    }
}
#endif
