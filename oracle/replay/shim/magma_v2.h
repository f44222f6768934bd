/* Stand-in for the MAGMA v2 interface used by the reference's RGF.H/Blas.H,
 * so that the unmodified reference sources compile and run on the host for
 * the CPU replay (test infrastructure only).  Declares the types, enums and
 * routines those headers name; only the double-precision routines RGF<double>
 * calls are defined (replay_shim.cpp), with host loops.  "Device" pointers
 * are host pointers. */
#ifndef RGF_REPLAY_MAGMA_V2_H
#define RGF_REPLAY_MAGMA_V2_H

#include <cuComplex.h>
#include <cuda_runtime_api.h>

typedef int magma_int_t;
typedef int magma_device_t;
typedef struct rgf_replay_queue* magma_queue_t;
typedef cuDoubleComplex magmaDoubleComplex;
typedef magmaDoubleComplex* magmaDoubleComplex_ptr;

typedef enum { MagmaNoTrans = 111, MagmaTrans = 112, MagmaConjTrans = 113 } magma_trans_t;
typedef enum { MagmaUpper = 121, MagmaLower = 122, MagmaFull = 123 } magma_uplo_t;
typedef enum { MagmaNonUnit = 131, MagmaUnit = 132 } magma_diag_t;
typedef enum { MagmaLeft = 141, MagmaRight = 142 } magma_side_t;

magma_trans_t magma_trans_const(char c);
magma_uplo_t magma_uplo_const(char c);
magma_diag_t magma_diag_const(char c);
magma_side_t magma_side_const(char c);

magma_int_t magma_init();
magma_int_t magma_finalize();
void magma_getdevice(magma_device_t* dev);
void magma_queue_create_from_cuda(magma_device_t dev, void* stream, void* cublas, void* cusparse,
                                  magma_queue_t* q);
void magma_queue_destroy(magma_queue_t q);
cudaStream_t magma_queue_get_cuda_stream(magma_queue_t q);
void* magma_queue_get_cublas_handle(magma_queue_t q);

void magma_dgemm(magma_trans_t ta, magma_trans_t tb, magma_int_t m, magma_int_t n, magma_int_t k,
                 double alpha, const double* A, magma_int_t lda, const double* B, magma_int_t ldb,
                 double beta, double* C, magma_int_t ldc, magma_queue_t q);
void magma_dtrsm(magma_side_t side, magma_uplo_t uplo, magma_trans_t trans, magma_diag_t diag,
                 magma_int_t m, magma_int_t n, double alpha, const double* A, magma_int_t lda,
                 double* B, magma_int_t ldb, magma_queue_t q);
magma_int_t magma_dpotrf_gpu(magma_uplo_t uplo, magma_int_t n, double* A, magma_int_t lda,
                             magma_int_t* info);
magma_int_t magma_dtrtri_gpu(magma_uplo_t uplo, magma_diag_t diag, magma_int_t n, double* A,
                             magma_int_t lda, magma_int_t* info);
void magmablas_dlacpy(magma_uplo_t uplo, magma_int_t m, magma_int_t n, const double* A,
                      magma_int_t lda, double* B, magma_int_t ldb, magma_queue_t q);

/* declared for the complex / LU wrappers in Blas.H; never called by the replay */
void magma_zgemm(magma_trans_t, magma_trans_t, magma_int_t, magma_int_t, magma_int_t,
                 magmaDoubleComplex, magmaDoubleComplex_ptr, magma_int_t, magmaDoubleComplex_ptr,
                 magma_int_t, magmaDoubleComplex, magmaDoubleComplex_ptr, magma_int_t,
                 magma_queue_t);
void magma_ztrsm(magma_side_t, magma_uplo_t, magma_trans_t, magma_diag_t, magma_int_t,
                 magma_int_t, magmaDoubleComplex, magmaDoubleComplex_ptr, magma_int_t,
                 magmaDoubleComplex_ptr, magma_int_t, magma_queue_t);
magma_int_t magma_zpotrf_gpu(magma_uplo_t, magma_int_t, magmaDoubleComplex_ptr, magma_int_t,
                             magma_int_t*);
magma_int_t magma_ztrtri_gpu(magma_uplo_t, magma_diag_t, magma_int_t, magmaDoubleComplex_ptr,
                             magma_int_t, magma_int_t*);
void magmablas_zlacpy(magma_uplo_t, magma_int_t, magma_int_t, magmaDoubleComplex_ptr,
                      magma_int_t, magmaDoubleComplex_ptr, magma_int_t, magma_queue_t);
magma_int_t magma_dgetrf_gpu(magma_int_t, magma_int_t, double*, magma_int_t, magma_int_t*,
                             magma_int_t*);
magma_int_t magma_zgetrf_gpu(magma_int_t, magma_int_t, magmaDoubleComplex_ptr, magma_int_t,
                             magma_int_t*, magma_int_t*);
magma_int_t magma_dgetrs_gpu(magma_trans_t, magma_int_t, magma_int_t, double*, magma_int_t,
                             magma_int_t*, double*, magma_int_t, magma_int_t*);
magma_int_t magma_zgetrs_gpu(magma_trans_t, magma_int_t, magma_int_t, magmaDoubleComplex_ptr,
                             magma_int_t, magma_int_t*, magmaDoubleComplex_ptr, magma_int_t,
                             magma_int_t*);
magma_int_t magma_dgesv_nopiv_gpu(magma_int_t, magma_int_t, double*, magma_int_t, double*,
                                  magma_int_t, magma_int_t*);
magma_int_t magma_zgesv_nopiv_gpu(magma_int_t, magma_int_t, magmaDoubleComplex_ptr, magma_int_t,
                                  magmaDoubleComplex_ptr, magma_int_t, magma_int_t*);
magma_int_t magma_dsysv_nopiv_gpu(magma_uplo_t, magma_int_t, magma_int_t, double*, magma_int_t,
                                  double*, magma_int_t, magma_int_t*);
magma_int_t magma_zhesv_nopiv_gpu(magma_uplo_t, magma_int_t, magma_int_t, magmaDoubleComplex_ptr,
                                  magma_int_t, magmaDoubleComplex_ptr, magma_int_t, magma_int_t*);
magma_int_t magma_dgetri_gpu(magma_int_t, double*, magma_int_t, magma_int_t*, double*,
                             magma_int_t, magma_int_t*);
magma_int_t magma_zgetri_gpu(magma_int_t, magmaDoubleComplex_ptr, magma_int_t, magma_int_t*,
                             magmaDoubleComplex_ptr, magma_int_t, magma_int_t*);
magma_int_t magma_zgetrf_nopiv_gpu(magma_int_t, magma_int_t, magmaDoubleComplex_ptr, magma_int_t,
                                   magma_int_t*);
magma_int_t magma_zgetrs_nopiv_gpu(magma_trans_t, magma_int_t, magma_int_t,
                                   magmaDoubleComplex_ptr, magma_int_t, magmaDoubleComplex_ptr,
                                   magma_int_t, magma_int_t*);

#endif
