/* Minimal stand-ins for the external libraries the reference's hot-path sources include
 * (MPI, SUNDIALS, RAJA, HDF5), so that src/utilities.cpp, src/euler3D.hpp and
 * src/raja_primordial_network.cpp compile unmodified on one rank with g++.
 *
 * TEST INFRASTRUCTURE ONLY: this builds the reference's own CPU code as a checker for the
 * oracle restatement and as a golden-vector generator.  Nothing in the product links it.
 *
 * Scope of each stand-in is exactly what those three files use:
 *  - MPI: one rank; Cartesian topology with periodic wrap to self; Isend/Irecv matched by tag
 *    through an in-process mailbox (the halo exchange in src/euler3D.hpp:577-791 sends to
 *    itself on a periodic axis); Bcast/Allreduce are identity on one rank.
 *  - SUNDIALS: realtype=double, a ManyVector-like N_Vector of up to 8 host arrays, a CSR
 *    SUNMatrix for the KLU (non-device) branch of calculate_jacobian_cvklu.
 *  - RAJA: serial forall.
 *  - HDF5: H5Fopen / H5LTread_dataset_double / H5Fclose over a reader for superblock-v0 files
 *    with contiguous float64 datasets (h5v0.c).
 */
#ifndef GBMV_REF_SHIM_CORE_H
#define GBMV_REF_SHIM_CORE_H

#include <stddef.h>
#include <string.h>
#include <stdlib.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------- SUNDIALS types ---------------- */
typedef double realtype;
typedef double sunrealtype;
typedef long sunindextype;
typedef int booleantype;
#define RCONST(x) x
#define SUNTRUE 1
#define SUNFALSE 0
#define SUNRsqrt(x) ((x) <= 0.0 ? 0.0 : sqrt((x)))

typedef void* SUNContext;
typedef void* SUNMemoryHelper;
int SUNContext_Create(void* comm, SUNContext* ctx);
int SUNContext_Free(SUNContext* ctx);
int SUNMemoryHelper_Destroy(SUNMemoryHelper h);

/* A ManyVector-like vector: nsub host arrays. */
struct shim_nvector {
  int nsub;
  double* sub[8];
  long len[8];
};
typedef struct shim_nvector* N_Vector;

double* N_VGetSubvectorArrayPointer_MPIManyVector(N_Vector v, int k);
/* a one-component view of component k (defined in shim_glue.c, for the main programs' glue) */
N_Vector N_VGetSubvector_MPIManyVector(N_Vector v, sunindextype k);
double* N_VGetArrayPointer(N_Vector v);
void N_VConst(double c, N_Vector v);

/* CSR matrix for the host (KLU) branch of the reference Jacobian. */
struct shim_sunmatrix {
  long N;
  long nnz;
  double* data;
  sunindextype* rowptrs;
  sunindextype* colvals;
};
typedef struct shim_sunmatrix* SUNMatrix;
double* SUNSparseMatrix_Data(SUNMatrix A);
sunindextype* SUNSparseMatrix_IndexPointers(SUNMatrix A);
sunindextype* SUNSparseMatrix_IndexValues(SUNMatrix A);
int SUNMatZero(SUNMatrix A);

typedef int ARKODE_ERKTableID;
typedef int ARKODE_DIRKTableID;
typedef int ARKODE_MRITableID;
#define ARKODE_ERK_NONE (-1)
#define ARKODE_DIRK_NONE (-1)
#define ARKODE_MRI_NONE (-1)

/* ---------------- MPI (one rank) ---------------- */
typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef int MPI_Request;
typedef struct { int MPI_SOURCE, MPI_TAG, MPI_ERROR; } MPI_Status;
#define MPI_SUCCESS 0
#define MPI_COMM_WORLD 0
#define MPI_PROC_NULL (-2)
#define MPI_REQUEST_NULL (-1)
#define MPI_DOUBLE 1
#define MPI_INT 2
#define MPI_LONG 3
#define MPI_SUNREALTYPE MPI_DOUBLE
#define MPI_MAX 1
#define MPI_MIN 2
#define MPI_SUM 3
#define MPI_IN_PLACE ((void*)1)

int MPI_Init(int* argc, char*** argv);
int MPI_Finalize(void);
int MPI_Abort(MPI_Comm comm, int code);
int MPI_Comm_size(MPI_Comm comm, int* n);
int MPI_Comm_rank(MPI_Comm comm, int* r);
int MPI_Dims_create(int nnodes, int ndims, int* dims);
int MPI_Cart_create(MPI_Comm old, int ndims, const int* dims, const int* periods, int reorder,
                    MPI_Comm* cart);
int MPI_Cart_get(MPI_Comm comm, int maxdims, int* dims, int* periods, int* coords);
int MPI_Cart_rank(MPI_Comm comm, const int* coords, int* rank);
int MPI_Irecv(void* buf, int count, MPI_Datatype t, int src, int tag, MPI_Comm comm,
              MPI_Request* req);
int MPI_Isend(const void* buf, int count, MPI_Datatype t, int dst, int tag, MPI_Comm comm,
              MPI_Request* req);
int MPI_Waitall(int n, MPI_Request* reqs, MPI_Status* stats);
int MPI_Bcast(void* buf, int count, MPI_Datatype t, int root, MPI_Comm comm);
int MPI_Allreduce(const void* sbuf, void* rbuf, int count, MPI_Datatype t, MPI_Op op,
                  MPI_Comm comm);
int MPI_Reduce(const void* sbuf, void* rbuf, int count, MPI_Datatype t, MPI_Op op, int root,
               MPI_Comm comm);
int MPI_Barrier(MPI_Comm comm);
double MPI_Wtime(void);

/* ---------------- HDF5 subset ---------------- */
typedef long hid_t;
typedef int herr_t;
#define H5F_ACC_RDONLY 0u
#define H5P_DEFAULT 0
hid_t H5Fopen(const char* name, unsigned flags, hid_t plist);
herr_t H5Fclose(hid_t id);
herr_t H5LTread_dataset_double(hid_t loc, const char* name, double* out);

#ifdef __cplusplus
}
#endif

#endif
