/*
 * minipetsc.c -- implementation of the PETSc stand-in declared in minipetsc.h: one rank,
 * DMDA views over plain arrays, Vec basics and a DMSwarm field registry.  Test infrastructure
 * (see minipetsc.h for the semantics kept from PETSc).
 */
#include "minipetsc.h"

#include <stdarg.h>
#include <time.h>

enum { OBJ_NONE = 0, OBJ_VEC, OBJ_DMDA, OBJ_SWARM, OBJ_RANDOM, OBJ_VIEWER };

#define MAX_VIEWS 16
#define MAX_FIELDS 32

typedef struct {
  char name[64];
  PetscInt bs;
  PetscDataType type;
  size_t esize;          /* bytes per point */
  unsigned char *data;   /* capacity * esize */
  int held;              /* outstanding DMSwarmGetField views */
} SwarmField;

struct _p_PetscObject {
  int kind;
  char name[64];
  PetscObjectState state;
  /* Vec */
  PetscScalar *data;
  PetscInt n, bs;
  DM dm;
  int borrowed;                        /* data belongs to a swarm field */
  void *views[MAX_VIEWS];              /* DMDA array views handed out (to free on restore) */
  void *view_key[MAX_VIEWS];
  /* DMDA */
  DMDALocalInfo info;
  DM cdm;
  Vec coords;
  Vec spare_local, spare_global;
  /* DMSwarm */
  SwarmField fields[MAX_FIELDS];
  int nfields, finalized;
  PetscInt npoints, capacity;
  DM celldm;
  DMSwarmType stype;
  /* PetscRandom */
  unsigned long long seed, rstate;
  PetscScalar lo, hi;
};

static char g_err[1024];

PetscErrorCode minipetsc_seterr(const char *func, const char *file, int line, PetscErrorCode code, const char *fmt,
                                ...) {
  if (!g_err[0]) {
    char msg[768];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(msg, sizeof msg, fmt, ap);
    va_end(ap);
    snprintf(g_err, sizeof g_err, "[%s %s:%d] %s", func, file, line, msg);
  }
  return code;
}
const char *minipetsc_last_error(void) { return g_err; }
void minipetsc_clear_error(void) { g_err[0] = 0; }

static PetscObject new_obj(int kind) {
  PetscObject o = (PetscObject)calloc(1, sizeof(struct _p_PetscObject));
  if (o) o->kind = kind;
  return o;
}

/* ---- MPI, one rank ---- */
static size_t dtype_size(MPI_Datatype t) { return (size_t)(t & 0xff); }
int MPI_Comm_rank(MPI_Comm comm, int *rank) { (void)comm; *rank = 0; return 0; }
int MPI_Comm_size(MPI_Comm comm, int *size) { (void)comm; *size = 1; return 0; }
int MPI_Allreduce(const void *send, void *recv, int count, MPI_Datatype type, MPI_Op op, MPI_Comm comm) {
  (void)op; (void)comm;
  if (send != MPI_IN_PLACE) memmove(recv, send, (size_t)count * dtype_size(type));
  return 0;
}
int MPI_Reduce(const void *send, void *recv, int count, MPI_Datatype type, MPI_Op op, int root, MPI_Comm comm) {
  (void)root;
  return MPI_Allreduce(send, recv, count, type, op, comm);
}
int MPI_Exscan(const void *send, void *recv, int count, MPI_Datatype type, MPI_Op op, MPI_Comm comm) {
  /* rank 0's result is undefined in MPI; zero it */
  (void)send; (void)op; (void)comm;
  memset(recv, 0, (size_t)count * dtype_size(type));
  return 0;
}
int MPI_Allgather(const void *send, int scount, MPI_Datatype stype, void *recv, int rcount, MPI_Datatype rtype,
                  MPI_Comm comm) {
  (void)rcount; (void)rtype; (void)comm;
  if (send != MPI_IN_PLACE) memmove(recv, send, (size_t)scount * dtype_size(stype));
  return 0;
}
int MPI_Gather(const void *send, int scount, MPI_Datatype stype, void *recv, int rcount, MPI_Datatype rtype,
               int root, MPI_Comm comm) {
  (void)root;
  return MPI_Allgather(send, scount, stype, recv, rcount, rtype, comm);
}
int MPI_Scatter(const void *send, int scount, MPI_Datatype stype, void *recv, int rcount, MPI_Datatype rtype,
                int root, MPI_Comm comm) {
  (void)rcount; (void)rtype; (void)root; (void)comm;
  if (recv != MPI_IN_PLACE) memmove(recv, send, (size_t)scount * dtype_size(stype));
  return 0;
}
int MPI_Bcast(void *buf, int count, MPI_Datatype type, int root, MPI_Comm comm) {
  (void)buf; (void)count; (void)type; (void)root; (void)comm;
  return 0;
}
int MPI_Barrier(MPI_Comm comm) { (void)comm; return 0; }
int MPI_Abort(MPI_Comm comm, int code) { (void)comm; fprintf(stderr, "MPI_Abort(%d)\n", code); abort(); }

/* ---- memory and sorting ---- */
PetscErrorCode minipetsc_malloc(size_t bytes, void **p, int zero) {
  *p = zero ? calloc(1, bytes ? bytes : 1) : malloc(bytes ? bytes : 1);
  return *p ? 0 : PETSC_ERR_MEM;
}
PetscErrorCode minipetsc_realloc(size_t bytes, void **p) {
  void *q = realloc(*p, bytes ? bytes : 1);
  if (!q) return PETSC_ERR_MEM;
  *p = q;
  return 0;
}
static int cmp_i64(const void *a, const void *b) {
  const int64_t x = *(const int64_t *)a, y = *(const int64_t *)b;
  return (x > y) - (x < y);
}
PetscErrorCode PetscSortInt64(PetscInt n, PetscInt64 x[]) { qsort(x, (size_t)n, sizeof(int64_t), cmp_i64); return 0; }
PetscErrorCode PetscSortInt(PetscInt n, PetscInt x[]) { qsort(x, (size_t)n, sizeof(int64_t), cmp_i64); return 0; }
PetscErrorCode PetscStrallocpy(const char s[], char *t[]) {
  *t = NULL;
  if (!s) return 0;
  *t = (char *)malloc(strlen(s) + 1);
  if (!*t) return PETSC_ERR_MEM;
  strcpy(*t, s);
  return 0;
}
PetscErrorCode PetscStrcmp(const char a[], const char b[], PetscBool *flg) {
  *flg = (a && b && !strcmp(a, b)) || (!a && !b) ? PETSC_TRUE : PETSC_FALSE;
  return 0;
}

/* ---- printing, options, timing (quiet unless MINIPETSC_VERBOSE is set) ---- */
static int verbose(void) { return getenv("MINIPETSC_VERBOSE") != NULL; }
PetscErrorCode PetscPrintf(MPI_Comm comm, const char fmt[], ...) {
  (void)comm;
  if (verbose()) { va_list ap; va_start(ap, fmt); vprintf(fmt, ap); va_end(ap); }
  return 0;
}
PetscErrorCode PetscSynchronizedPrintf(MPI_Comm comm, const char fmt[], ...) {
  (void)comm;
  if (verbose()) { va_list ap; va_start(ap, fmt); vprintf(fmt, ap); va_end(ap); }
  return 0;
}
PetscErrorCode PetscSynchronizedFlush(MPI_Comm comm, FILE *fd) { (void)comm; (void)fd; return 0; }
PetscErrorCode PetscFPrintf(MPI_Comm comm, FILE *fd, const char fmt[], ...) {
  (void)comm;
  if (verbose()) { va_list ap; va_start(ap, fmt); vfprintf(fd, fmt, ap); va_end(ap); }
  return 0;
}
PetscErrorCode PetscSNPrintf(char *str, size_t len, const char fmt[], ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(str, len, fmt, ap);
  va_end(ap);
  return 0;
}
PetscErrorCode PetscInfo(PetscObject obj, const char fmt[], ...) { (void)obj; (void)fmt; return 0; }
PetscErrorCode PetscTime(PetscLogDouble *t) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  *t = (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
  return 0;
}
PetscErrorCode PetscLogEventRegister(const char name[], PetscClassId cid, PetscLogEvent *e) {
  (void)name; (void)cid; *e = 0; return 0;
}
PetscErrorCode PetscLogEventBegin(PetscLogEvent e, PetscObject a, PetscObject b, PetscObject c, PetscObject d) {
  (void)e; (void)a; (void)b; (void)c; (void)d; return 0;
}
PetscErrorCode PetscLogEventEnd(PetscLogEvent e, PetscObject a, PetscObject b, PetscObject c, PetscObject d) {
  (void)e; (void)a; (void)b; (void)c; (void)d; return 0;
}
PetscErrorCode PetscOptionsGetInt(void *o, const char p[], const char n[], PetscInt *v, PetscBool *set) {
  (void)o; (void)p; (void)n; (void)v; if (set) *set = PETSC_FALSE; return 0;
}
PetscErrorCode PetscOptionsGetReal(void *o, const char p[], const char n[], PetscReal *v, PetscBool *set) {
  (void)o; (void)p; (void)n; (void)v; if (set) *set = PETSC_FALSE; return 0;
}
PetscErrorCode PetscOptionsGetBool(void *o, const char p[], const char n[], PetscBool *v, PetscBool *set) {
  (void)o; (void)p; (void)n; (void)v; if (set) *set = PETSC_FALSE; return 0;
}
PetscErrorCode PetscOptionsGetString(void *o, const char p[], const char n[], char v[], size_t len, PetscBool *set) {
  (void)o; (void)p; (void)n; (void)v; (void)len; if (set) *set = PETSC_FALSE; return 0;
}
PetscErrorCode PetscOptionsHasName(void *o, const char p[], const char n[], PetscBool *set) {
  (void)o; (void)p; (void)n; if (set) *set = PETSC_FALSE; return 0;
}
PetscErrorCode PetscOptionsInsertFile(MPI_Comm comm, void *o, const char f[], PetscBool req) {
  (void)comm; (void)o; (void)f; (void)req; return PETSC_ERR_SUP;
}
PetscErrorCode PetscTestFile(const char name[], char mode, PetscBool *flg) {
  (void)mode;
  FILE *f = fopen(name, "r");
  *flg = f ? PETSC_TRUE : PETSC_FALSE;
  if (f) fclose(f);
  return 0;
}
PetscErrorCode PetscBarrier(PetscObject obj) { (void)obj; return 0; }

/* ---- objects ---- */
PetscErrorCode PetscObjectSetName(PetscObject obj, const char name[]) {
  if (!obj) return PETSC_ERR_ARG_NULL;
  snprintf(obj->name, sizeof obj->name, "%s", name ? name : "");
  return 0;
}
PetscErrorCode PetscObjectGetName(PetscObject obj, const char *name[]) {
  if (!obj) return PETSC_ERR_ARG_NULL;
  *name = obj->name;
  return 0;
}
PetscErrorCode PetscObjectGetComm(PetscObject obj, MPI_Comm *comm) { (void)obj; *comm = PETSC_COMM_WORLD; return 0; }
MPI_Comm PetscObjectComm(PetscObject obj) { (void)obj; return PETSC_COMM_WORLD; }
PetscErrorCode PetscObjectStateGet(PetscObject obj, PetscObjectState *state) {
  if (!obj) return PETSC_ERR_ARG_NULL;
  *state = obj->state;
  return 0;
}

/* ---- Vec ---- */
PetscErrorCode minipetsc_vec_create(DM dm, PetscInt n, PetscInt bs, Vec *v) {
  Vec x = new_obj(OBJ_VEC);
  if (!x) return PETSC_ERR_MEM;
  x->n = n;
  x->bs = bs > 0 ? bs : 1;
  x->dm = dm;
  x->data = (PetscScalar *)calloc((size_t)(n > 0 ? n : 1), sizeof(PetscScalar));
  if (!x->data) { free(x); return PETSC_ERR_MEM; }
  *v = x;
  return 0;
}
PetscScalar *minipetsc_vec_data(Vec v) { return v ? v->data : NULL; }
PetscInt minipetsc_vec_length(Vec v) { return v ? v->n : 0; }
void minipetsc_vec_touch(Vec v) { if (v) v->state++; }

PetscErrorCode VecCreate(MPI_Comm comm, Vec *v) { (void)comm; return minipetsc_vec_create(NULL, 0, 1, v); }
PetscErrorCode VecCreateSeq(MPI_Comm comm, PetscInt n, Vec *v) { (void)comm; return minipetsc_vec_create(NULL, n, 1, v); }
PetscErrorCode VecSetSizes(Vec v, PetscInt n, PetscInt N) {
  if (!v || v->kind != OBJ_VEC || v->borrowed) return PETSC_ERR_ARG_WRONGSTATE;
  const PetscInt m = n >= 0 ? n : N;
  PetscScalar *d = (PetscScalar *)realloc(v->data, (size_t)(m > 0 ? m : 1) * sizeof(PetscScalar));
  if (!d) return PETSC_ERR_MEM;
  memset(d, 0, (size_t)(m > 0 ? m : 1) * sizeof(PetscScalar));
  v->data = d;
  v->n = m;
  return 0;
}
PetscErrorCode VecSetBlockSize(Vec v, PetscInt bs) { v->bs = bs; return 0; }
PetscErrorCode VecSetFromOptions(Vec v) { (void)v; return 0; }
PetscErrorCode VecDuplicate(Vec v, Vec *w) {
  if (!v) return PETSC_ERR_ARG_NULL;
  return minipetsc_vec_create(v->dm, v->n, v->bs, w);
}
PetscErrorCode VecDestroy(Vec *v) {
  if (!v || !*v) return 0;
  if (!(*v)->borrowed) free((*v)->data);
  for (int q = 0; q < MAX_VIEWS; ++q) free((*v)->views[q]);
  free(*v);
  *v = NULL;
  return 0;
}
PetscErrorCode VecCopy(Vec x, Vec y) {
  if (!x || !y || x->n != y->n) return PETSC_ERR_ARG_SIZ;
  memcpy(y->data, x->data, (size_t)x->n * sizeof(PetscScalar));
  y->state++;
  return 0;
}
PetscErrorCode VecSet(Vec v, PetscScalar a) {
  if (!v) return PETSC_ERR_ARG_NULL;
  for (PetscInt q = 0; q < v->n; ++q) v->data[q] = a;
  v->state++;
  return 0;
}
PetscErrorCode VecZeroEntries(Vec v) { return VecSet(v, 0.0); }
PetscErrorCode VecGetSize(Vec v, PetscInt *n) { *n = v->n; return 0; }
PetscErrorCode VecGetLocalSize(Vec v, PetscInt *n) { *n = v->n; return 0; }
PetscErrorCode VecGetBlockSize(Vec v, PetscInt *bs) { *bs = v->bs; return 0; }
PetscErrorCode VecGetDM(Vec v, DM *dm) { *dm = v->dm; return 0; }
PetscErrorCode VecGetArray(Vec v, PetscScalar **a) { *a = v->data; return 0; }
PetscErrorCode VecRestoreArray(Vec v, PetscScalar **a) { v->state++; if (a) *a = NULL; return 0; }
PetscErrorCode VecGetArrayRead(Vec v, const PetscScalar **a) { *a = v->data; return 0; }
PetscErrorCode VecRestoreArrayRead(Vec v, const PetscScalar **a) { (void)v; if (a) *a = NULL; return 0; }
PetscErrorCode VecAssemblyBegin(Vec v) { (void)v; return 0; }
PetscErrorCode VecAssemblyEnd(Vec v) { (void)v; return 0; }
PetscErrorCode VecSum(Vec v, PetscScalar *s) {
  PetscScalar t = 0.0;
  for (PetscInt q = 0; q < v->n; ++q) t += v->data[q];
  *s = t;
  return 0;
}
PetscErrorCode VecMean(Vec v, PetscScalar *m) {
  PetscScalar t;
  VecSum(v, &t);
  *m = v->n ? t / (PetscScalar)v->n : 0.0;
  return 0;
}
PetscErrorCode VecMax(Vec v, PetscInt *idx, PetscReal *m) {
  PetscReal b = PETSC_MIN_REAL;
  PetscInt at = -1;
  for (PetscInt q = 0; q < v->n; ++q)
    if (v->data[q] > b) { b = v->data[q]; at = q; }
  if (idx) *idx = at;
  *m = b;
  return 0;
}
PetscErrorCode VecMin(Vec v, PetscInt *idx, PetscReal *m) {
  PetscReal b = PETSC_MAX_REAL;
  PetscInt at = -1;
  for (PetscInt q = 0; q < v->n; ++q)
    if (v->data[q] < b) { b = v->data[q]; at = q; }
  if (idx) *idx = at;
  *m = b;
  return 0;
}
PetscErrorCode VecNorm(Vec v, NormType t, PetscReal *nrm) {
  PetscReal s = 0.0;
  for (PetscInt q = 0; q < v->n; ++q) {
    const PetscReal a = fabs(v->data[q]);
    if (t == NORM_1) s += a;
    else if (t == NORM_INFINITY) s = a > s ? a : s;
    else s += a * a;
  }
  *nrm = (t == NORM_2 || t == NORM_FROBENIUS) ? sqrt(s) : s;
  return 0;
}
PetscErrorCode VecView(Vec v, PetscViewer viewer) { (void)v; (void)viewer; return 0; }
PetscErrorCode VecLoad(Vec v, PetscViewer viewer) { (void)v; (void)viewer; return PETSC_ERR_SUP; }
PetscErrorCode VecAXPY(Vec y, PetscScalar a, Vec x) {
  for (PetscInt q = 0; q < y->n; ++q) y->data[q] += a * x->data[q];
  y->state++;
  return 0;
}
PetscErrorCode VecScale(Vec v, PetscScalar a) {
  for (PetscInt q = 0; q < v->n; ++q) v->data[q] *= a;
  v->state++;
  return 0;
}

PetscErrorCode PetscViewerBinaryOpen(MPI_Comm comm, const char name[], PetscFileMode mode, PetscViewer *viewer) {
  (void)comm; (void)name; (void)mode; *viewer = NULL; return PETSC_ERR_SUP;
}
PetscErrorCode PetscViewerDestroy(PetscViewer *viewer) { if (viewer) *viewer = NULL; return 0; }

/* ---- random numbers: a rand48 stream ---- */
PetscErrorCode PetscRandomCreate(MPI_Comm comm, PetscRandom *r) {
  (void)comm;
  *r = new_obj(OBJ_RANDOM);
  if (!*r) return PETSC_ERR_MEM;
  (*r)->hi = 1.0;
  return 0;
}
PetscErrorCode PetscRandomSetType(PetscRandom r, PetscRandomType type) { (void)r; (void)type; return 0; }
PetscErrorCode PetscRandomSetInterval(PetscRandom r, PetscScalar lo, PetscScalar hi) { r->lo = lo; r->hi = hi; return 0; }
PetscErrorCode PetscRandomSetSeed(PetscRandom r, unsigned long seed) { r->seed = seed; return 0; }
PetscErrorCode PetscRandomSeed(PetscRandom r) { r->rstate = ((unsigned long long)r->seed << 16) | 0x330e; return 0; }
PetscErrorCode PetscRandomGetValueReal(PetscRandom r, PetscReal *v) {
  r->rstate = (r->rstate * 0x5deece66dull + 0xbull) & ((1ull << 48) - 1);
  *v = r->lo + (r->hi - r->lo) * ((double)r->rstate / 281474976710656.0);
  return 0;
}
PetscErrorCode PetscRandomGetValue(PetscRandom r, PetscScalar *v) { return PetscRandomGetValueReal(r, v); }
PetscErrorCode PetscRandomSetFromOptions(PetscRandom r) { (void)r; return 0; }
PetscErrorCode PetscRandomDestroy(PetscRandom *r) { if (r && *r) { free(*r); *r = NULL; } return 0; }

/* ---- DM / DMDA ---- */
PetscErrorCode DMCreate(MPI_Comm comm, DM *dm) {
  (void)comm;
  *dm = new_obj(OBJ_NONE);
  return *dm ? 0 : PETSC_ERR_MEM;
}
PetscErrorCode DMSetType(DM dm, DMType type) {
  if (!dm) return PETSC_ERR_ARG_NULL;
  if (!strcmp(type, DMSWARM)) dm->kind = OBJ_SWARM;
  else if (!strcmp(type, DMDA)) dm->kind = OBJ_DMDA;
  else return PETSC_ERR_SUP;
  return 0;
}
PetscErrorCode DMSetDimension(DM dm, PetscInt dim) { (void)dm; (void)dim; return 0; }
PetscErrorCode DMSetFromOptions(DM dm) { (void)dm; return 0; }
PetscErrorCode DMSetUp(DM dm) { (void)dm; return 0; }
PetscErrorCode DMView(DM dm, PetscViewer viewer) { (void)dm; (void)viewer; return 0; }
PetscErrorCode DMDestroy(DM *dm) {
  if (!dm || !*dm) return 0;
  DM d = *dm;
  if (d->kind == OBJ_SWARM)
    for (int f = 0; f < d->nfields; ++f) free(d->fields[f].data);
  VecDestroy(&d->spare_local);
  VecDestroy(&d->spare_global);
  free(d);
  *dm = NULL;
  return 0;
}

PetscErrorCode minipetsc_dmda_create(PetscInt M, PetscInt N, PetscInt P, PetscInt dof, DM *da) {
  DM d = new_obj(OBJ_DMDA);
  if (!d) return PETSC_ERR_MEM;
  DMDALocalInfo *i = &d->info;
  i->da = d;
  i->dim = 3; i->dof = dof; i->sw = 1;
  i->mx = M; i->my = N; i->mz = P;
  i->xs = 0; i->ys = 0; i->zs = 0; i->xm = M; i->ym = N; i->zm = P;
  i->gxs = 0; i->gys = 0; i->gzs = 0; i->gxm = M; i->gym = N; i->gzm = P;
  i->bx = i->by = i->bz = DM_BOUNDARY_NONE;
  i->st = DMDA_STENCIL_BOX;
  *da = d;
  return 0;
}
PetscErrorCode DMDACreate3d(MPI_Comm comm, DMBoundaryType bx, DMBoundaryType by, DMBoundaryType bz,
                            DMDAStencilType st, PetscInt M, PetscInt N, PetscInt P, PetscInt m, PetscInt n,
                            PetscInt p, PetscInt dof, PetscInt s, const PetscInt lx[], const PetscInt ly[],
                            const PetscInt lz[], DM *da) {
  (void)comm; (void)m; (void)n; (void)p; (void)lx; (void)ly; (void)lz;
  if (bx != DM_BOUNDARY_NONE || by != DM_BOUNDARY_NONE || bz != DM_BOUNDARY_NONE) return PETSC_ERR_SUP;
  PetscErrorCode e = minipetsc_dmda_create(M, N, P, dof, da);
  if (!e) { (*da)->info.sw = s; (*da)->info.st = st; }
  return e;
}
PetscErrorCode minipetsc_dm_set_coordinates(DM da, DM cdm, Vec coords) {
  if (!da) return PETSC_ERR_ARG_NULL;
  da->cdm = cdm;
  da->coords = coords;
  return 0;
}
static PetscErrorCode need_dmda(DM da) { return (da && da->kind == OBJ_DMDA) ? 0 : PETSC_ERR_ARG_WRONG; }
PetscErrorCode DMDAGetLocalInfo(DM da, DMDALocalInfo *info) {
  PetscErrorCode e = need_dmda(da);
  if (e) return e;
  *info = da->info;
  return 0;
}
PetscErrorCode DMDAGetInfo(DM da, PetscInt *dim, PetscInt *M, PetscInt *N, PetscInt *P, PetscInt *m, PetscInt *n,
                           PetscInt *p, PetscInt *dof, PetscInt *s, DMBoundaryType *bx, DMBoundaryType *by,
                           DMBoundaryType *bz, DMDAStencilType *st) {
  PetscErrorCode e = need_dmda(da);
  if (e) return e;
  const DMDALocalInfo *i = &da->info;
  if (dim) *dim = i->dim;
  if (M) *M = i->mx;
  if (N) *N = i->my;
  if (P) *P = i->mz;
  if (m) *m = 1;
  if (n) *n = 1;
  if (p) *p = 1;
  if (dof) *dof = i->dof;
  if (s) *s = i->sw;
  if (bx) *bx = i->bx;
  if (by) *by = i->by;
  if (bz) *bz = i->bz;
  if (st) *st = i->st;
  return 0;
}
PetscErrorCode DMDAGetCorners(DM da, PetscInt *x, PetscInt *y, PetscInt *z, PetscInt *m, PetscInt *n, PetscInt *p) {
  PetscErrorCode e = need_dmda(da);
  if (e) return e;
  const DMDALocalInfo *i = &da->info;
  if (x) *x = i->xs;
  if (y) *y = i->ys;
  if (z) *z = i->zs;
  if (m) *m = i->xm;
  if (n) *n = i->ym;
  if (p) *p = i->zm;
  return 0;
}
PetscErrorCode DMDAGetGhostCorners(DM da, PetscInt *x, PetscInt *y, PetscInt *z, PetscInt *m, PetscInt *n,
                                   PetscInt *p) {
  PetscErrorCode e = need_dmda(da);
  if (e) return e;
  const DMDALocalInfo *i = &da->info;
  if (x) *x = i->gxs;
  if (y) *y = i->gys;
  if (z) *z = i->gzs;
  if (m) *m = i->gxm;
  if (n) *n = i->gym;
  if (p) *p = i->gzm;
  return 0;
}
PetscErrorCode DMDAGetNeighbors(DM da, const PetscMPIInt *ranks[]) {
  static const PetscMPIInt nb[27] = {-1, -1, -1, -1, -1, -1, -1, -1, -1, -1, -1, -1, -1, 0,
                                     -1, -1, -1, -1, -1, -1, -1, -1, -1, -1, -1, -1, -1};
  (void)da;
  *ranks = nb;
  return 0;
}
PetscErrorCode DMDASetNumProcs(DM da, PetscInt m, PetscInt n, PetscInt p) { (void)da; (void)m; (void)n; (void)p; return 0; }

/* [k][j][i] view with global indices: planes[k] -> rows[j] -> element 0 of the row; for the
 * DOF form one more level of pointers, per point, to its components. */
static PetscErrorCode make_view(DM da, Vec v, void *array, int dof_form) {
  PetscErrorCode e = need_dmda(da);
  if (e) return e;
  if (!v || !array) return PETSC_ERR_ARG_NULL;
  const DMDALocalInfo *i = &da->info;
  const PetscInt dof = i->dof;
  if (v->n != i->gxm * i->gym * i->gzm * dof) return PETSC_ERR_ARG_INCOMP;
  int slot = -1;
  for (int q = 0; q < MAX_VIEWS; ++q)
    if (!v->views[q]) { slot = q; break; }
  if (slot < 0) return PETSC_ERR_ARG_WRONGSTATE;
  const size_t nplanes = (size_t)i->gzm, nrows = (size_t)(i->gzm * i->gym);
  const size_t npts = dof_form ? (size_t)(i->gzm * i->gym * i->gxm) : 0;
  void **mem = (void **)malloc((nplanes + nrows + npts + 1) * sizeof(void *));
  if (!mem) return PETSC_ERR_MEM;
  PetscScalar ***planes = (PetscScalar ***)mem;
  PetscScalar **rows = (PetscScalar **)(mem + nplanes);
  PetscScalar **pts = (PetscScalar **)(mem + nplanes + nrows);
  for (PetscInt k = 0; k < i->gzm; ++k) {
    for (PetscInt j = 0; j < i->gym; ++j) {
      PetscScalar *row0 = v->data + ((k * i->gym + j) * i->gxm) * dof;
      if (dof_form) {
        PetscScalar **prow = pts + (k * i->gym + j) * i->gxm;
        for (PetscInt x = 0; x < i->gxm; ++x) prow[x] = row0 + x * dof;
        rows[k * i->gym + j] = (PetscScalar *)(prow - i->gxs);
      } else {
        rows[k * i->gym + j] = row0 - i->gxs * dof;
      }
    }
    planes[k] = rows + k * i->gym - i->gys;
  }
  void *handle = (void *)(planes - i->gzs);
  v->views[slot] = mem;
  v->view_key[slot] = handle;
  *(void **)array = handle;
  return 0;
}
static PetscErrorCode drop_view(Vec v, void *array, int wrote) {
  if (!v || !array) return PETSC_ERR_ARG_NULL;
  void *handle = *(void **)array;
  for (int q = 0; q < MAX_VIEWS; ++q)
    if (v->views[q] && v->view_key[q] == handle) {
      free(v->views[q]);
      v->views[q] = NULL;
      v->view_key[q] = NULL;
      *(void **)array = NULL;
      if (wrote) v->state++;
      return 0;
    }
  return PETSC_ERR_ARG_WRONGSTATE;
}
PetscErrorCode DMDAVecGetArray(DM da, Vec v, void *a) { return make_view(da, v, a, 0); }
PetscErrorCode DMDAVecRestoreArray(DM da, Vec v, void *a) { (void)da; return drop_view(v, a, 1); }
PetscErrorCode DMDAVecGetArrayRead(DM da, Vec v, void *a) { return make_view(da, v, a, 0); }
PetscErrorCode DMDAVecRestoreArrayRead(DM da, Vec v, void *a) { (void)da; return drop_view(v, a, 0); }
PetscErrorCode DMDAVecGetArrayDOF(DM da, Vec v, void *a) { return make_view(da, v, a, 1); }
PetscErrorCode DMDAVecRestoreArrayDOF(DM da, Vec v, void *a) { (void)da; return drop_view(v, a, 1); }
PetscErrorCode DMDAVecGetArrayDOFRead(DM da, Vec v, void *a) { return make_view(da, v, a, 1); }
PetscErrorCode DMDAVecRestoreArrayDOFRead(DM da, Vec v, void *a) { (void)da; return drop_view(v, a, 0); }

PetscErrorCode DMGetCoordinateDM(DM dm, DM *cdm) {
  if (!dm || !dm->cdm) return PETSC_ERR_ARG_WRONGSTATE;
  *cdm = dm->cdm;
  return 0;
}
PetscErrorCode DMGetCoordinates(DM dm, Vec *c) {
  if (!dm) return PETSC_ERR_ARG_NULL;
  *c = dm->coords;
  return 0;
}
PetscErrorCode DMGetCoordinatesLocal(DM dm, Vec *c) { return DMGetCoordinates(dm, c); }
static PetscInt dmda_len(DM dm) { return dm->info.gxm * dm->info.gym * dm->info.gzm * dm->info.dof; }
PetscErrorCode DMCreateGlobalVector(DM dm, Vec *v) {
  PetscErrorCode e = need_dmda(dm);
  if (e) return e;
  return minipetsc_vec_create(dm, dmda_len(dm), dm->info.dof, v);
}
PetscErrorCode DMCreateLocalVector(DM dm, Vec *v) { return DMCreateGlobalVector(dm, v); }
PetscErrorCode DMGetLocalVector(DM dm, Vec *v) { return DMCreateGlobalVector(dm, v); }
PetscErrorCode DMRestoreLocalVector(DM dm, Vec *v) { (void)dm; return VecDestroy(v); }
PetscErrorCode DMGetGlobalVector(DM dm, Vec *v) { return DMCreateGlobalVector(dm, v); }
PetscErrorCode DMRestoreGlobalVector(DM dm, Vec *v) { (void)dm; return VecDestroy(v); }
/* one rank, no ghost points outside the grid: local and global vectors hold the same values */
static PetscErrorCode move(Vec from, InsertMode mode, Vec to) {
  if (!from || !to || from->n != to->n) return PETSC_ERR_ARG_SIZ;
  if (mode == ADD_VALUES)
    for (PetscInt q = 0; q < to->n; ++q) to->data[q] += from->data[q];
  else
    memcpy(to->data, from->data, (size_t)to->n * sizeof(PetscScalar));
  to->state++;
  return 0;
}
PetscErrorCode DMGlobalToLocal(DM dm, Vec g, InsertMode mode, Vec l) { (void)dm; return move(g, mode, l); }
PetscErrorCode DMGlobalToLocalBegin(DM dm, Vec g, InsertMode mode, Vec l) { (void)dm; return move(g, mode, l); }
PetscErrorCode DMGlobalToLocalEnd(DM dm, Vec g, InsertMode mode, Vec l) { (void)dm; (void)g; (void)mode; (void)l; return 0; }
PetscErrorCode DMLocalToGlobal(DM dm, Vec l, InsertMode mode, Vec g) { (void)dm; return move(l, mode, g); }
PetscErrorCode DMLocalToGlobalBegin(DM dm, Vec l, InsertMode mode, Vec g) { (void)dm; return move(l, mode, g); }
PetscErrorCode DMLocalToGlobalEnd(DM dm, Vec l, InsertMode mode, Vec g) { (void)dm; (void)l; (void)mode; (void)g; return 0; }

/* ---- DMSwarm ---- */
const char *const PetscDataTypes[] = {"UNKNOWN", "DOUBLE", "COMPLEX", "LONG", "SHORT", "FLOAT", "CHAR", "LOGICAL",
                                      "ENUM", "BOOL", "__FLOAT128", "OBJECT", "FUNCTION", "STRING", "__FP16",
                                      "STRUCT", "INT", "INT64", "COUNT", "PetscDataType", "PETSC_", NULL};
static size_t type_size(PetscDataType t) {
  switch (t) {
    case PETSC_DOUBLE: return sizeof(double);
    case PETSC_INT: return sizeof(PetscInt);
    case PETSC_INT64: return sizeof(int64_t);
    case PETSC_FLOAT: return sizeof(float);
    case PETSC_CHAR: return 1;
    case PETSC_SHORT: return sizeof(short);
    case PETSC_LONG: return sizeof(long);
    case PETSC_BOOL: return sizeof(PetscBool);
    default: return 0;
  }
}
static PetscErrorCode need_swarm(DM dm) { return (dm && dm->kind == OBJ_SWARM) ? 0 : PETSC_ERR_ARG_WRONG; }
static SwarmField *find_field(DM dm, const char *name) {
  for (int f = 0; f < dm->nfields; ++f)
    if (!strcmp(dm->fields[f].name, name)) return &dm->fields[f];
  return NULL;
}
PetscErrorCode DMSwarmSetType(DM dm, DMSwarmType type) { PetscErrorCode e = need_swarm(dm); if (!e) dm->stype = type; return e; }
PetscErrorCode DMSwarmSetCellDM(DM dm, DM cell) { PetscErrorCode e = need_swarm(dm); if (!e) dm->celldm = cell; return e; }
PetscErrorCode DMSwarmRegisterPetscDatatypeField(DM dm, const char name[], PetscInt bs, PetscDataType type) {
  PetscErrorCode e = need_swarm(dm);
  if (e) return e;
  if (dm->finalized) SETERRQ(PETSC_COMM_SELF, PETSC_ERR_ARG_WRONGSTATE, "field registration is finalized");
  if (find_field(dm, name)) SETERRQ(PETSC_COMM_SELF, PETSC_ERR_ARG_WRONG, "field %s already registered", name);
  if (dm->nfields == MAX_FIELDS || !type_size(type) || bs < 1) return PETSC_ERR_SUP;
  SwarmField *f = &dm->fields[dm->nfields++];
  memset(f, 0, sizeof *f);
  snprintf(f->name, sizeof f->name, "%s", name);
  f->bs = bs;
  f->type = type;
  f->esize = (size_t)bs * type_size(type);
  return 0;
}
PetscErrorCode DMSwarmFinalizeFieldRegister(DM dm) {
  PetscErrorCode e = need_swarm(dm);
  if (e) return e;
  if (dm->finalized) return 0;
  if (!find_field(dm, DMSwarmField_pid)) CHKERRQ(DMSwarmRegisterPetscDatatypeField(dm, DMSwarmField_pid, 1, PETSC_INT64));
  if (!find_field(dm, DMSwarmField_rank)) CHKERRQ(DMSwarmRegisterPetscDatatypeField(dm, DMSwarmField_rank, 1, PETSC_INT));
  dm->finalized = 1;
  return 0;
}
static PetscErrorCode reserve_points(DM dm, PetscInt cap) {
  if (cap <= dm->capacity) return 0;
  for (int f = 0; f < dm->nfields; ++f) {
    SwarmField *fl = &dm->fields[f];
    unsigned char *d = (unsigned char *)realloc(fl->data, (size_t)cap * fl->esize);
    if (!d) return PETSC_ERR_MEM;
    memset(d + (size_t)dm->capacity * fl->esize, 0, (size_t)(cap - dm->capacity) * fl->esize);
    fl->data = d;
  }
  dm->capacity = cap;
  return 0;
}
PetscErrorCode DMSwarmSetLocalSizes(DM dm, PetscInt n, PetscInt buffer) {
  PetscErrorCode e = need_swarm(dm);
  if (e) return e;
  if (!dm->finalized) SETERRQ(PETSC_COMM_SELF, PETSC_ERR_ARG_WRONGSTATE, "field registration not finalized");
  CHKERRQ(reserve_points(dm, n + (buffer > 0 ? buffer : 0)));
  dm->npoints = n;
  return 0;
}
PetscErrorCode DMSwarmGetLocalSize(DM dm, PetscInt *n) {
  PetscErrorCode e = need_swarm(dm);
  if (e) return e;
  *n = dm->npoints;
  return 0;
}
PetscErrorCode DMSwarmGetSize(DM dm, PetscInt *n) { return DMSwarmGetLocalSize(dm, n); }
PetscErrorCode DMSwarmGetField(DM dm, const char name[], PetscInt *bs, PetscDataType *type, void **data) {
  PetscErrorCode e = need_swarm(dm);
  if (e) return e;
  SwarmField *f = find_field(dm, name);
  if (!f) SETERRQ(PETSC_COMM_SELF, PETSC_ERR_ARG_UNKNOWN, "no swarm field %s", name);
  if (f->held) SETERRQ(PETSC_COMM_SELF, PETSC_ERR_ARG_WRONGSTATE, "swarm field %s is already held", name);
  if (bs) *bs = f->bs;
  if (type) *type = f->type;
  if (data) *data = f->data;
  f->held = 1;
  return 0;
}
PetscErrorCode DMSwarmRestoreField(DM dm, const char name[], PetscInt *bs, PetscDataType *type, void **data) {
  PetscErrorCode e = need_swarm(dm);
  if (e) return e;
  SwarmField *f = find_field(dm, name);
  if (!f) SETERRQ(PETSC_COMM_SELF, PETSC_ERR_ARG_UNKNOWN, "no swarm field %s", name);
  if (!f->held) SETERRQ(PETSC_COMM_SELF, PETSC_ERR_ARG_WRONGSTATE, "swarm field %s is not held", name);
  f->held = 0;
  if (bs) *bs = f->bs;
  if (type) *type = f->type;
  if (data) *data = NULL;
  return 0;
}
int minipetsc_swarm_fields_held(DM dm) {
  int h = 0;
  if (dm && dm->kind == OBJ_SWARM)
    for (int f = 0; f < dm->nfields; ++f) h += dm->fields[f].held;
  return h;
}
PetscErrorCode DMSwarmAddNPoints(DM dm, PetscInt n) {
  PetscErrorCode e = need_swarm(dm);
  if (e) return e;
  if (dm->npoints + n > dm->capacity) CHKERRQ(reserve_points(dm, 2 * (dm->npoints + n)));
  for (int f = 0; f < dm->nfields; ++f)
    memset(dm->fields[f].data + (size_t)dm->npoints * dm->fields[f].esize, 0, (size_t)n * dm->fields[f].esize);
  dm->npoints += n;
  return 0;
}
PetscErrorCode DMSwarmAddPoint(DM dm) { return DMSwarmAddNPoints(dm, 1); }
PetscErrorCode DMSwarmRemovePoint(DM dm) {
  PetscErrorCode e = need_swarm(dm);
  if (e) return e;
  if (dm->npoints > 0) dm->npoints--;
  return 0;
}
PetscErrorCode DMSwarmRemovePointAtIndex(DM dm, PetscInt idx) {
  PetscErrorCode e = need_swarm(dm);
  if (e) return e;
  if (idx < 0 || idx >= dm->npoints) SETERRQ(PETSC_COMM_SELF, PETSC_ERR_ARG_OUTOFRANGE, "index %lld out of range", (long long)idx);
  for (int f = 0; f < dm->nfields; ++f)
    if (dm->fields[f].held) SETERRQ(PETSC_COMM_SELF, PETSC_ERR_ARG_WRONGSTATE, "swarm field %s is held", dm->fields[f].name);
  const PetscInt last = dm->npoints - 1;
  if (idx != last)
    for (int f = 0; f < dm->nfields; ++f) {
      SwarmField *fl = &dm->fields[f];
      memcpy(fl->data + (size_t)idx * fl->esize, fl->data + (size_t)last * fl->esize, fl->esize);
    }
  dm->npoints--;
  return 0;
}
PetscErrorCode DMSwarmMigrate(DM dm, PetscBool remove_sent) { (void)dm; (void)remove_sent; return PETSC_ERR_SUP; }
static PetscErrorCode field_vec(DM dm, const char name[], Vec *v) {
  PetscErrorCode e = need_swarm(dm);
  if (e) return e;
  SwarmField *f = find_field(dm, name);
  if (!f) SETERRQ(PETSC_COMM_SELF, PETSC_ERR_ARG_UNKNOWN, "no swarm field %s", name);
  if (f->type != PETSC_DOUBLE) SETERRQ(PETSC_COMM_SELF, PETSC_ERR_SUP, "swarm field %s is not real", name);
  Vec x = new_obj(OBJ_VEC);
  if (!x) return PETSC_ERR_MEM;
  x->data = (PetscScalar *)f->data;
  x->n = dm->npoints * f->bs;
  x->bs = f->bs;
  x->borrowed = 1;
  *v = x;
  return 0;
}
PetscErrorCode DMSwarmCreateGlobalVectorFromField(DM dm, const char name[], Vec *v) { return field_vec(dm, name, v); }
PetscErrorCode DMSwarmDestroyGlobalVectorFromField(DM dm, const char name[], Vec *v) { (void)dm; (void)name; return VecDestroy(v); }
PetscErrorCode DMSwarmCreateLocalVectorFromField(DM dm, const char name[], Vec *v) { return field_vec(dm, name, v); }
PetscErrorCode DMSwarmDestroyLocalVectorFromField(DM dm, const char name[], Vec *v) { (void)dm; (void)name; return VecDestroy(v); }
PetscErrorCode DMSwarmVectorDefineField(DM dm, const char name[]) { (void)dm; (void)name; return 0; }
