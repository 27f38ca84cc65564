/* Stand-in for the one PETSc call the reference makes (oracle build only). */
#ifndef FFV_STUB_PETSC_H
#define FFV_STUB_PETSC_H
int PetscInitialize(int *argc, char ***argv, const char *file, const char *help);
#endif
