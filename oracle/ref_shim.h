/*
 * ref_shim.h - pre-included (gcc -include) when oracle/Makefile compiles the
 * reference's own C path (Heterogeneous_MHD/C/*.c of pandaPQY/MHD-GPU) from
 * the sources where they lie.  TEST INFRASTRUCTURE ONLY.
 *
 * The reference sizes its static pencil scratch and its full-grid advect
 * temporary from a compile-time box size (Heterogeneous_MHD/C/parameter.h:6-11,
 * fluidx.c:9-15, advectbyzx.c:7).  Defining the PARAMETER_H guard here makes
 * the reference's parameter.h a no-op and replaces those sizes with maxima, so
 * one build serves every box of up to 512 cells per pencil and 2^25 cells.
 * System headers are pulled in first so the size macros cannot reach them.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>
#include <assert.h>

#define PARAMETER_H
#define box_nx 512
#define box_ny 512
#define box_nz 128
#define TOTAL_CELL_NUMBER box_nx*box_ny*box_nz
#define nu 5
#define nb 3

typedef struct {
  float *u;
  float *b;
  int nx;
  int ny;
  int nz;
  float dt;
  int total_cell_number;
  int no_meaning;
} variable_context;
