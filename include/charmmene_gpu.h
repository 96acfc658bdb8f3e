/*
 * charmmene_gpu.h — the reference's Fortran/C energy interface (src/FORTRAN_interface.cpp:23-106,
 * library libcharmmene) backed by the GB300 engine: libcharmmene_gpu.so exports the same seven
 * symbols with the same arguments, so a program linked against libcharmmene links against this
 * library instead with no source change.
 *
 * Differences from the reference, all on failure paths: a bad input prints the reason to stderr
 * and exits with a negative code, as the reference's readers do; the reference would crash or
 * read garbage on the same inputs.  Strings are NUL-terminated C strings, as the reference
 * assumes.  One system per process (file-scope state, like the reference).
 */
#ifndef CHARMMENE_GPU_H
#define CHARMMENE_GPU_H

#ifdef __cplusplus
extern "C" {
#endif

/* PerConditions(type, a, b, c, alpha, beta, gamma): type "none", "cubic" or "orbic". */
void set_pbc_(char* type, double* a, double* b, double* c, double* alpha, double* beta, double* gamma);
/* Ens_NVT(natom, volume, T). */
void set_ens_(int* natom, double* Temp);
/* FField (cut mode "full" or "switch", cutoff, cuton, skin) + IO_MDBAS(COR_file, FF_file) +
 * List_nonBonded: builds the device system in plain FP64 with its exclusion and Verlet lists. */
void set_ff_and_cor_(char* cutoffmode, double* ctoff, double* cton, double* dcut, char* FF_file, char* COR_file);
/* FField::getE(ener) in kcal/mol: [tot, pot, kin, elec, vdw, bond, ang, ub, dihe, impr]. */
void get_energy_(double ener[10]);
/* AtomList::setCoords for every atom. */
void set_coords_(double x[], double y[], double z[]);
void get_mass_(double mass[]);
void clean_(void);

#ifdef __cplusplus
}
#endif

#endif
