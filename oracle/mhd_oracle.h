/*
 * mhd_oracle.h - CPU restatement of the reference C path of Pen's relaxing TVD
 * MHD step (Heterogeneous_MHD/C/*.c of pandaPQY/MHD-GPU).
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker for the CUDA kernels
 * in mhd-gpu_gb300/csrc.  Only tests/, __graft_entry__.smoke() and the CPU
 * baseline leg of bench.py may load it.  Nothing in the product links it.
 *
 * Two builds of the same source live in liboracle.so:
 *   oracle_*    real = float   (bit-exact restatement of the reference C path,
 *                               including its C promotions of 2.0-style literals
 *                               to double; compiled with -ffp-contract=off)
 *   oracle64_*  real = double  (the same solver in FP64; equals the reference
 *                               sources compiled with -Dfloat=double)
 *
 * Arrays use the reference layout: u(5,nx,ny,nz), b(3,nx,ny,nz), component
 * fastest, then i, j, k (Heterogeneous_MHD/C/array_definition.h:12-14).
 *
 * The subroutine entry points keep the reference signatures
 * (Heterogeneous_MHD/C/spu_function.h:1-15) so that a test can call the
 * oracle and the reference compiled from its own sources on identical inputs.
 */
#ifndef MHD_ORACLE_H
#define MHD_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* float build */
void  oracle_fluidx(float *u, float *b, int *nx, int *ny, int *nz, float *dt,
                    float *update_u, float *update_b, int iter);
void  oracle_advectbyzx(float *u, float *b, int *nx, int *ny, int *nz, float *dt,
                        float *update_u, float *update_b);
void  oracle_transpose12(float *u, float *b, float *update_u, float *update_b,
                         int *nx, int *ny, int *nz, int iter);
void  oracle_transpose13(float *u, float *b, float *update_u, float *update_b,
                         int *nx, int *ny, int *nz);
float oracle_calcfl(float *u, float *b, int *nx, int *ny, int *nz);
float oracle_calcfl_averaged(float *u, float *b, int *nx, int *ny, int *nz);
void  oracle_copy_matrix(float *u, float *b, int *nx, int *ny, int *nz,
                         float *update_u, float *update_b);
float oracle_dt_from_cfl(float inv_c, double cfl_number, float t, float tf);
void  oracle_step(float *u, float *b, int nx, int ny, int nz, float dt,
                  float *work_u, float *work_b);
int   oracle_run(float *u, float *b, int nx, int ny, int nz, double cfl_number,
                 int cfl_mode, float *t, float tf, int max_steps, float *dt_log);

/* double build */
void   oracle64_fluidx(double *u, double *b, int *nx, int *ny, int *nz, double *dt,
                       double *update_u, double *update_b, int iter);
void   oracle64_advectbyzx(double *u, double *b, int *nx, int *ny, int *nz, double *dt,
                           double *update_u, double *update_b);
void   oracle64_transpose12(double *u, double *b, double *update_u, double *update_b,
                            int *nx, int *ny, int *nz, int iter);
void   oracle64_transpose13(double *u, double *b, double *update_u, double *update_b,
                            int *nx, int *ny, int *nz);
double oracle64_calcfl(double *u, double *b, int *nx, int *ny, int *nz);
double oracle64_calcfl_averaged(double *u, double *b, int *nx, int *ny, int *nz);
void   oracle64_copy_matrix(double *u, double *b, int *nx, int *ny, int *nz,
                            double *update_u, double *update_b);
double oracle64_dt_from_cfl(double inv_c, double cfl_number, double t, double tf);
void   oracle64_step(double *u, double *b, int nx, int ny, int nz, double dt,
                     double *work_u, double *work_b);
int    oracle64_run(double *u, double *b, int nx, int ny, int nz, double cfl_number,
                    int cfl_mode, double *t, double tf, int max_steps, double *dt_log);

/* OpenMP thread count for the pencil loops (1 = the reference's serial C path).
 * Results are bit-identical for every thread count on NaN-free inputs. */
void oracle_set_threads(int nthreads);
int  oracle_get_threads(void);

#ifdef __cplusplus
}
#endif
#endif
