/*
 * Test driver for the reference REMD server's exchange sweep (src/Server.c:145-192,
 * `rearrange`).  Linked with the reference Server.c (its main renamed).  Reads from
 * stdin:
 *     seed n rounds
 *     then `rounds` blocks of n lines "num T E"   (replica slot i: temperature index,
 *                                                   temperature, potential energy)
 * Each block overwrites the slots' energies (and, in the first block only, the
 * temperatures), calls rearrange() once and prints n lines "num T" (hex T).
 * srand(seed) is called once, like the server's main (src/Server.c:57).
 */
#include <stdio.h>
#include <stdlib.h>

struct REMDTempStr { int num; double T; };
extern double **probability;
void rearrange(double *Epot, struct REMDTempStr *T, int number_of_connects);

int sdmd_ref_rand(void) { return rand(); }

int main(void) {
    long seed; int n, rounds;
    if (scanf("%ld %d %d", &seed, &n, &rounds) != 3) return 2;
    srand(seed);
    probability = (double **)calloc(n, sizeof(double *));
    for (int i = 0; i < n; i++) probability[i] = (double *)calloc(2, sizeof(double));
    struct REMDTempStr *T = calloc(n, sizeof(*T));
    double *E = calloc(n, sizeof(double));
    for (int r = 0; r < rounds; r++) {
        for (int i = 0; i < n; i++) {
            int num; double t, e;
            if (scanf("%d %lf %lf", &num, &t, &e) != 3) return 2;
            if (r == 0) { T[i].num = num; T[i].T = t; }
            E[i] = e;
        }
        rearrange(E, T, n);
        for (int i = 0; i < n; i++) printf("%d %a\n", T[i].num, T[i].T);
    }
    return 0;
}
