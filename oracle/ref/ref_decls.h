/* Declarations that the reference's inputset.c (lines 47-56) uses but strdata.h does
 * not provide; force-included into that one translation unit by oracle/ref/Makefile. */
extern double NDFI_DIST_SOLID_0, NDFI_DIST_SOLID_1, NDFI_DIST_SOLID_2, NDFI_DIST_SOLID_3;
