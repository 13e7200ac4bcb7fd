/* One-rank implementations behind shim_core.h (test infrastructure only). */
#include "shim_core.h"

#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <time.h>

/* ---------------- SUNDIALS pieces ---------------- */
int SUNContext_Create(void* comm, SUNContext* ctx) { (void)comm; *ctx = (void*)1; return 0; }
int SUNContext_Free(SUNContext* ctx) { *ctx = NULL; return 0; }
int SUNMemoryHelper_Destroy(SUNMemoryHelper h) { (void)h; return 0; }

double* N_VGetSubvectorArrayPointer_MPIManyVector(N_Vector v, int k) {
  if (!v || k < 0 || k >= v->nsub) return NULL;
  return v->sub[k];
}
double* N_VGetArrayPointer(N_Vector v) { return v ? v->sub[0] : NULL; }
void N_VConst(double c, N_Vector v) {
  for (int s = 0; s < v->nsub; ++s)
    for (long i = 0; i < v->len[s]; ++i) v->sub[s][i] = c;
}

double* SUNSparseMatrix_Data(SUNMatrix A) { return A->data; }
sunindextype* SUNSparseMatrix_IndexPointers(SUNMatrix A) { return A->rowptrs; }
sunindextype* SUNSparseMatrix_IndexValues(SUNMatrix A) { return A->colvals; }
int SUNMatZero(SUNMatrix A) {
  memset(A->data, 0, sizeof(double) * (size_t)A->nnz);
  return 0;
}

/* ---------------- MPI, one rank ---------------- */
int MPI_Init(int* argc, char*** argv) { (void)argc; (void)argv; return MPI_SUCCESS; }
int MPI_Finalize(void) { return MPI_SUCCESS; }
int MPI_Abort(MPI_Comm comm, int code) {
  (void)comm;
  fprintf(stderr, "shim MPI_Abort(%d)\n", code);
  abort();
}
int MPI_Comm_size(MPI_Comm comm, int* n) { (void)comm; *n = 1; return MPI_SUCCESS; }
int MPI_Comm_rank(MPI_Comm comm, int* r) { (void)comm; *r = 0; return MPI_SUCCESS; }
int MPI_Dims_create(int nnodes, int ndims, int* dims) {
  (void)nnodes;
  for (int i = 0; i < ndims; ++i) dims[i] = 1;
  return MPI_SUCCESS;
}
static int g_periods[3];
int MPI_Cart_create(MPI_Comm old, int ndims, const int* dims, const int* periods, int reorder,
                    MPI_Comm* cart) {
  (void)old; (void)dims; (void)reorder;
  for (int i = 0; i < ndims && i < 3; ++i) g_periods[i] = periods[i];
  *cart = 0;
  return MPI_SUCCESS;
}
int MPI_Cart_get(MPI_Comm comm, int maxdims, int* dims, int* periods, int* coords) {
  (void)comm;
  for (int i = 0; i < maxdims; ++i) { dims[i] = 1; periods[i] = g_periods[i]; coords[i] = 0; }
  return MPI_SUCCESS;
}
int MPI_Cart_rank(MPI_Comm comm, const int* coords, int* rank) {
  (void)comm;
  for (int i = 0; i < 3; ++i)
    if (coords[i] != 0 && !g_periods[i]) { *rank = MPI_PROC_NULL; return MPI_SUCCESS; }
  *rank = 0;
  return MPI_SUCCESS;
}

/* Tag-matched self messaging: receives are posted before sends in the reference's
 * ExchangeStart, but both orders are handled. */
#define SHIM_MAXMSG 64
typedef struct { void* buf; const void* sbuf; int count; int tag; int is_recv; int live; } shim_msg;
static shim_msg g_msgs[SHIM_MAXMSG];

static int elsize(MPI_Datatype t) { return t == MPI_INT ? (int)sizeof(int) : t == MPI_LONG ? (int)sizeof(long) : (int)sizeof(double); }

int MPI_Irecv(void* buf, int count, MPI_Datatype t, int src, int tag, MPI_Comm comm,
              MPI_Request* req) {
  (void)src; (void)comm;
  for (int i = 0; i < SHIM_MAXMSG; ++i)
    if (g_msgs[i].live && !g_msgs[i].is_recv && g_msgs[i].tag == tag) {
      memcpy(buf, g_msgs[i].sbuf, (size_t)count * elsize(t));
      free((void*)g_msgs[i].sbuf);
      g_msgs[i].live = 0;
      *req = MPI_REQUEST_NULL;
      return MPI_SUCCESS;
    }
  for (int i = 0; i < SHIM_MAXMSG; ++i)
    if (!g_msgs[i].live) {
      g_msgs[i] = (shim_msg){buf, NULL, count * elsize(t), tag, 1, 1};
      *req = i;
      return MPI_SUCCESS;
    }
  return 1;
}
int MPI_Isend(const void* buf, int count, MPI_Datatype t, int dst, int tag, MPI_Comm comm,
              MPI_Request* req) {
  (void)dst; (void)comm;
  size_t nb = (size_t)count * elsize(t);
  for (int i = 0; i < SHIM_MAXMSG; ++i)
    if (g_msgs[i].live && g_msgs[i].is_recv && g_msgs[i].tag == tag) {
      memcpy(g_msgs[i].buf, buf, nb);
      g_msgs[i].live = 0;
      *req = MPI_REQUEST_NULL;
      return MPI_SUCCESS;
    }
  for (int i = 0; i < SHIM_MAXMSG; ++i)
    if (!g_msgs[i].live) {
      void* copy = malloc(nb);
      memcpy(copy, buf, nb);
      g_msgs[i] = (shim_msg){NULL, copy, (int)nb, tag, 0, 1};
      *req = MPI_REQUEST_NULL;
      return MPI_SUCCESS;
    }
  return 1;
}
int MPI_Waitall(int n, MPI_Request* reqs, MPI_Status* stats) {
  (void)stats;
  for (int i = 0; i < n; ++i)
    if (reqs[i] != MPI_REQUEST_NULL && g_msgs[reqs[i]].live) {
      fprintf(stderr, "shim MPI_Waitall: unmatched receive tag %d\n", g_msgs[reqs[i]].tag);
      return 1;
    }
  return MPI_SUCCESS;
}
int MPI_Bcast(void* buf, int count, MPI_Datatype t, int root, MPI_Comm comm) {
  (void)buf; (void)count; (void)t; (void)root; (void)comm;
  return MPI_SUCCESS;
}
int MPI_Allreduce(const void* sbuf, void* rbuf, int count, MPI_Datatype t, MPI_Op op,
                  MPI_Comm comm) {
  (void)op; (void)comm;
  if (sbuf != MPI_IN_PLACE) memcpy(rbuf, sbuf, (size_t)count * elsize(t));
  return MPI_SUCCESS;
}
int MPI_Reduce(const void* sbuf, void* rbuf, int count, MPI_Datatype t, MPI_Op op, int root,
               MPI_Comm comm) {
  (void)root;
  return MPI_Allreduce(sbuf, rbuf, count, t, op, comm);
}
int MPI_Barrier(MPI_Comm comm) { (void)comm; return MPI_SUCCESS; }
double MPI_Wtime(void) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

/* ---------------- HDF5 superblock-v0 reader ---------------- */
typedef struct { unsigned char* d; size_t n; } h5file;
#define H5MAXF 4
static h5file g_h5[H5MAXF];

static uint64_t rd64(const unsigned char* p) { uint64_t v = 0; for (int i = 7; i >= 0; --i) v = (v << 8) | p[i]; return v; }
static uint32_t rd32(const unsigned char* p) { return (uint32_t)p[0] | ((uint32_t)p[1] << 8) | ((uint32_t)p[2] << 16) | ((uint32_t)p[3] << 24); }
static uint16_t rd16(const unsigned char* p) { return (uint16_t)(p[0] | (p[1] << 8)); }

hid_t H5Fopen(const char* name, unsigned flags, hid_t plist) {
  (void)flags; (void)plist;
  FILE* f = fopen(name, "rb");
  if (!f) return -1;
  fseek(f, 0, SEEK_END);
  long n = ftell(f);
  fseek(f, 0, SEEK_SET);
  unsigned char* d = (unsigned char*)malloc((size_t)n);
  if (fread(d, 1, (size_t)n, f) != (size_t)n) { fclose(f); free(d); return -1; }
  fclose(f);
  static const unsigned char sig[8] = {0x89, 'H', 'D', 'F', '\r', '\n', 0x1a, '\n'};
  if (n < 96 || memcmp(d, sig, 8) != 0 || d[8] != 0 || d[13] != 8 || d[14] != 8) { free(d); return -1; }
  for (int i = 0; i < H5MAXF; ++i)
    if (!g_h5[i].d) { g_h5[i].d = d; g_h5[i].n = (size_t)n; return i + 1; }
  free(d);
  return -1;
}
herr_t H5Fclose(hid_t id) {
  if (id < 1 || id > H5MAXF) return -1;
  free(g_h5[id - 1].d);
  g_h5[id - 1].d = NULL;
  return 0;
}

/* Walks the root group (B-tree -> SNOD entries, names in the local heap) for `name`. */
static long h5_find(const h5file* f, const char* name) {
  const unsigned char* d = f->d;
  const unsigned char* root = d + 24 + 32;              /* root symbol table entry */
  uint64_t btree = rd64(root + 24), heap = rd64(root + 32);
  if (memcmp(d + heap, "HEAP", 4) != 0) return -1;
  uint64_t heapdata = rd64(d + heap + 24);
  uint64_t stack[64]; int sp = 0; stack[sp++] = btree;
  while (sp) {
    uint64_t node = stack[--sp];
    if (memcmp(d + node, "TREE", 4) != 0 || d[node + 4] != 0) return -1;
    int level = d[node + 5], nused = rd16(d + node + 6);
    const unsigned char* p = d + node + 24 + 8;          /* after header + key0 */
    for (int c = 0; c < nused; ++c, p += 16) {
      uint64_t child = rd64(p);
      if (level > 0) { if (sp < 64) stack[sp++] = child; continue; }
      if (memcmp(d + child, "SNOD", 4) != 0) return -1;
      int nsym = rd16(d + child + 6);
      for (int s = 0; s < nsym; ++s) {
        const unsigned char* e = d + child + 8 + 40 * s;
        const char* nm = (const char*)(d + heapdata + rd64(e));
        if (strcmp(nm, name) == 0) return (long)rd64(e + 8);
      }
    }
  }
  return -1;
}

herr_t H5LTread_dataset_double(hid_t loc, const char* name, double* out) {
  if (loc < 1 || loc > H5MAXF || !g_h5[loc - 1].d) return -1;
  const h5file* f = &g_h5[loc - 1];
  const unsigned char* d = f->d;
  if (name[0] == '/') ++name;
  long oh = h5_find(f, name);
  if (oh < 0 || d[oh] != 1) return -1;
  int nmsg = rd16(d + oh + 2);
  uint64_t blk_start[8], blk_size[8]; int nblk = 1, seen = 0;
  blk_start[0] = (uint64_t)oh + 16; blk_size[0] = rd32(d + oh + 8);
  uint64_t nelem = 0, addr = 0; int have_dims = 0, have_layout = 0;
  for (int b = 0; b < nblk && seen < nmsg; ++b) {
    uint64_t p = blk_start[b], end = blk_start[b] + blk_size[b];
    while (p + 8 <= end && seen < nmsg) {
      int mtype = rd16(d + p), msize = rd16(d + p + 2);
      const unsigned char* body = d + p + 8;
      ++seen;
      if (mtype == 0x10 && nblk < 8) { blk_start[nblk] = rd64(body); blk_size[nblk] = rd64(body + 8); ++nblk; }
      else if (mtype == 0x01) {
        int ver = body[0], ndim = body[1];
        const unsigned char* q = body + (ver == 1 ? 8 : 4);
        nelem = 1;
        for (int i = 0; i < ndim; ++i) nelem *= rd64(q + 8 * i);
        have_dims = 1;
      } else if (mtype == 0x03) {
        if ((body[0] & 0x0F) != 1 || rd32(body + 4) != 8 || (body[1] & 1)) return -1;
      } else if (mtype == 0x08) {
        if (body[0] == 3) { if (body[1] != 1) return -1; addr = rd64(body + 2); have_layout = 1; }
        else if (body[0] == 1 || body[0] == 2) { if (body[2] != 1) return -1; addr = rd64(body + 8); have_layout = 1; }
        else return -1;
      } else if (mtype == 0x0B) {
        return -1;
      }
      p += 8 + (uint64_t)msize;
    }
  }
  if (!have_dims || !have_layout || addr + nelem * 8 > f->n) return -1;
  memcpy(out, d + addr, nelem * 8);
  return 0;
}
