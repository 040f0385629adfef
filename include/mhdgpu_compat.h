/*
 * mhdgpu_compat.h - the reference C path's subroutine API, served by the
 * sm_103a kernels of libmhdgpu.so.
 *
 * Same names, signatures and argument meaning as
 * Heterogeneous_MHD/C/spu_function.h:1-15 of pandaPQY/MHD-GPU: host pointers,
 * sizes by pointer, (u, b) written from (update_u, update_b).  Each call copies
 * its inputs to the GPU, runs the kernel and copies the result back before it
 * returns.  A driver written for the reference links against these unchanged.
 *
 * Differences from the reference, all additive:
 *   - transpose13 accepts nx != nz (the reference prints "nz<>nx not
 *     supported" and leaves the output untouched, C/transpose13.c:58-61);
 *   - errors are printed to stderr and kept in mhdgpu_compat_status()
 *     instead of being silent.
 */
#ifndef MHDGPU_COMPAT_H
#define MHDGPU_COMPAT_H

#ifdef __cplusplus
extern "C" {
#endif

void fluidx(float *u, float *b, int *nx, int *ny, int *nz, float *dt, float *update_u,
            float *update_b, int iter);
void advectbyzx(float *u, float *b, int *nx, int *ny, int *nz, float *dt, float *update_u,
                float *update_b);
void transpose12(float *u, float *b, float *update_u, float *update_b, int *nx, int *ny, int *nz,
                 int iter);
void transpose13(float *u, float *b, float *update_u, float *update_b, int *nx, int *ny, int *nz);
float calcfl(float *u, float *b, int *nx, int *ny, int *nz);
void copy_matrix(float *u, float *b, int *nx, int *ny, int *nz, float *update_u, float *update_b);

/* status of the last compat call on this thread (MHD_OK or an MHD_ERR_* code) */
int mhdgpu_compat_status(void);

#ifdef __cplusplus
}
#endif

#endif /* MHDGPU_COMPAT_H */
