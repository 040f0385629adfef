/* mhdgpu_fortran.h - the Fortran original's subroutines (OpenMP/mhd.f90:
 * 249-474) with gfortran's external names: lower case with a trailing
 * underscore, every argument by reference.  The main loop of mhd.f90:41-72,
 * compiled against libmhdgpu.so, runs on the GPU unchanged:
 *
 *   call fluidx(u,b,nx,ny,nz,dt)           -> fluidx_
 *   call advectbyzx(u,b,nx,ny,nz,dt)       -> advectbyzx_
 *   call transpose12(ut,bt,u,b,nx,ny,nz)   -> transpose12_  (ut may be u)
 *   call transpose13(ut,bt,u,b,nx,ny,nz)   -> transpose13_  (ut may be u)
 *   dt = 0.9*cfl(u,b)                      -> cfl_(u,b,nx,ny,nz): the program's
 *        internal function made external, so it takes the sizes; release 0.2
 *        CFL formula (B averaged to the cell centre), returns 1/c.
 *
 * Host arrays u(5,nx,ny,nz) and b(3,nx,ny,nz) in Fortran order (the
 * reference layout); each call uploads, runs the sm_103a kernel and
 * downloads, like the compat entries of mhdgpu_compat.h, whose device
 * buffers and status (mhdgpu_compat_status) they share.  The arithmetic is
 * the C path's (Heterogeneous_MHD/C/), which rounds b_x's flux updates in a
 * fixed order; the Fortran advectbyzx applies them in its loop order, with
 * OpenMP threads racing on b(1,:,jm,k) (mhd.f90:284-286).
 */
#ifndef MHDGPU_FORTRAN_H
#define MHDGPU_FORTRAN_H

#ifdef __cplusplus
extern "C" {
#endif

void fluidx_(float *u, float *b, int *nx, int *ny, int *nz, float *dt);
void advectbyzx_(float *u, float *b, int *nx, int *ny, int *nz, float *dt);
void transpose12_(float *ut, float *bt, float *u, float *b, int *nx, int *ny, int *nz);
void transpose13_(float *ut, float *bt, float *u, float *b, int *nx, int *ny, int *nz);
float cfl_(float *u, float *b, int *nx, int *ny, int *nz);

#ifdef __cplusplus
}
#endif

#endif /* MHDGPU_FORTRAN_H */
