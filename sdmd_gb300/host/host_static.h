/*
 * host_static.h -- private to the host library: the static records of a built
 * system that the engine does not use but the reference's checkpoint holds
 * (PropertyStr's extra properties, the residue and peptide tables, the
 * force-field name), so savedata.c can write savedData.dat for a new run.
 */
#ifndef SDMD_HOST_STATIC_H
#define SDMD_HOST_STATIC_H

#include "sdmd_host.h"

typedef struct sdmd_host_static {
    int32_t n_aa, n_prot;
    const char *names, *resnames;          /* 8 bytes per atom */
    const char *ext;                       /* 32 bytes per atom: extraProperty[2][16] */
    const char *aa_name;                   /* 8 bytes per residue 0..n_aa */
    const int32_t *aa_type, *aa_start, *aa_end, *aa_prot;
    const double *aa_mass;
    const int32_t *pep_start, *pep_end, *pep_aa_start, *pep_aa_end;   /* 0..n_prot */
    const double *pep_mass;
    const char *method;                    /* the Force_Field word, 20 bytes */
    const double *mass0;                   /* atom 0's mass and type (FindTargetAtom) */
    const int32_t *type0;
    const double *hbpot;                   /* HBPotential: BB_r BB_v SS_r SS_v BS_r BS_v */
    const double *charge;                  /* InitializeCharge's, per atom */
    const char *wall_name, *wall_ext;      /* a smooth wall's Wall.txt record: name (8), extraProperty (2 x 16) */
    double wall_lib_mass;                  /* and its mass (obstruction walls' atoms are the same record) */
} sdmd_host_static;

void sdmd_host_static_info(const sdmd_host_system *h, sdmd_host_static *out);

#endif
