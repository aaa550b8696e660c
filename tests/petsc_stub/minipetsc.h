/*
 * minipetsc.h -- a small stand-in for the part of PETSc (3.19, 64-bit PetscInt) that the
 * particle path of PICurv and this library's reference-signature shim use: the scalar and
 * handle types, the error macros, one-rank MPI, DMDA local arrays, Vec basics and the DMSwarm
 * field registry.  Test infrastructure: it lets the reference's own C sources and the shim
 * compile and run on a machine without PETSc or MPI, with one rank owning the whole grid.
 *
 * Semantics kept from PETSc because results depend on them:
 *   - DMDAVecGetArray / DMDAVecGetArrayRead return [k][j][i] views indexed with global
 *     indices (one rank: ghosted range = whole grid);
 *   - DMSwarmRemovePointAtIndex moves the last point into the removed slot, field by field;
 *   - DMSwarmFinalizeFieldRegister adds the built-in fields "DMSwarm_pid" (PETSC_INT64) and
 *     "DMSwarm_rank" (PETSC_INT);
 *   - error macros return the code up the call chain (SETERRQ / CHKERRQ / PetscCall).
 * Everything else a PETSc routine might do (logging, options, viewers, migration between ranks)
 * is either a no-op or returns PETSC_ERR_SUP.
 */
#ifndef MINIPETSC_H
#define MINIPETSC_H

#include <stddef.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- scalar and handle types ---- */
typedef int PetscErrorCode;
typedef int64_t PetscInt;      /* the reference's PETSc is built with 64-bit indices */
typedef int64_t PetscInt64;
typedef int PetscMPIInt;
typedef double PetscReal;
typedef double PetscScalar;
typedef double PetscLogDouble;
typedef int PetscLogEvent;
typedef int PetscClassId;
#define PETSC_OBJECT_CLASSID ((PetscClassId)0)
typedef enum { PETSC_FALSE = 0, PETSC_TRUE = 1 } PetscBool;
typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;

typedef struct _p_PetscObject *PetscObject;
typedef struct _p_PetscObject *DM;
typedef struct _p_PetscObject *Vec;
typedef struct _p_PetscObject *PetscRandom;
typedef struct _p_PetscObject *PetscViewer;
typedef struct _p_PetscObject *PF;
typedef const char *DMType;
typedef const char *PetscRandomType;
typedef const char *PetscViewerType;
typedef long long PetscObjectState;

typedef enum { PETSC_DATATYPE_UNKNOWN = 0, PETSC_DOUBLE = 1, PETSC_COMPLEX = 2, PETSC_LONG = 3, PETSC_SHORT = 4,
               PETSC_FLOAT = 5, PETSC_CHAR = 6, PETSC_BIT_LOGICAL = 7, PETSC_ENUM = 8, PETSC_BOOL = 9,
               PETSC___FLOAT128 = 10, PETSC_OBJECT = 11, PETSC_FUNCTION = 12, PETSC_STRING = 13,
               PETSC___FP16 = 14, PETSC_STRUCT = 15, PETSC_INT = 16, PETSC_INT64 = 17, PETSC_COUNT = 18 } PetscDataType;
#define PETSC_REAL PETSC_DOUBLE
#define PETSC_SCALAR PETSC_DOUBLE
extern const char *const PetscDataTypes[];
#define PetscInt_FMT "lld"
#define PetscInt64_FMT "lld"

typedef enum { NOT_SET_VALUES, INSERT_VALUES, ADD_VALUES, MAX_VALUES, MIN_VALUES } InsertMode;
typedef enum { DM_BOUNDARY_NONE, DM_BOUNDARY_GHOSTED, DM_BOUNDARY_MIRROR, DM_BOUNDARY_PERIODIC,
               DM_BOUNDARY_TWIST } DMBoundaryType;
typedef enum { DMDA_STENCIL_STAR, DMDA_STENCIL_BOX } DMDAStencilType;
typedef enum { DMSWARM_BASIC = 0, DMSWARM_PIC } DMSwarmType;
typedef enum { DMSWARM_MIGRATE_BASIC = 0 } DMSwarmMigrateType;
typedef enum { FILE_MODE_UNDEFINED = -1, FILE_MODE_READ = 0, FILE_MODE_WRITE, FILE_MODE_APPEND } PetscFileMode;
typedef enum { NORM_1 = 0, NORM_2 = 1, NORM_FROBENIUS = 2, NORM_INFINITY = 3 } NormType;

typedef struct {
  DM da;
  PetscInt dim, dof, sw;
  PetscInt mx, my, mz;          /* global numbers of grid points */
  PetscInt xs, ys, zs;          /* first owned point */
  PetscInt xm, ym, zm;          /* owned widths */
  PetscInt gxs, gys, gzs;       /* first ghosted point */
  PetscInt gxm, gym, gzm;       /* ghosted widths */
  DMBoundaryType bx, by, bz;
  DMDAStencilType st;
} DMDALocalInfo;

#define DMDA "da"
#define DMSWARM "swarm"
#define PETSCRAND48 "rand48"
#define PETSCRAND "rand"
#define PETSCVIEWERBINARY "binary"

/* ---- communicators (one rank) ---- */
#define MPI_COMM_SELF ((MPI_Comm)1)
#define MPI_COMM_WORLD ((MPI_Comm)2)
#define PETSC_COMM_SELF MPI_COMM_SELF
#define PETSC_COMM_WORLD MPI_COMM_WORLD
#define MPI_PROC_NULL (-2)
#define MPI_SUCCESS 0
#define MPI_BYTE ((MPI_Datatype)1)
#define MPI_CHAR ((MPI_Datatype)1)
#define MPI_INT ((MPI_Datatype)4)
#define MPI_LONG ((MPI_Datatype)8)
#define MPI_LONG_LONG ((MPI_Datatype)8)
#define MPI_INT64_T ((MPI_Datatype)8)
#define MPI_DOUBLE ((MPI_Datatype)0x108)
#define MPIU_INT MPI_INT64_T
#define MPIU_INT64 MPI_INT64_T
#define MPIU_REAL MPI_DOUBLE
#define MPIU_SCALAR MPI_DOUBLE
#define MPIU_BOOL MPI_INT
#define MPI_SUM ((MPI_Op)1)
#define MPI_MAX ((MPI_Op)2)
#define MPI_MIN ((MPI_Op)3)
#define MPIU_SUM MPI_SUM
#define MPIU_MAX MPI_MAX
#define MPIU_MIN MPI_MIN
#define MPI_IN_PLACE ((void *)1)
int MPI_Comm_rank(MPI_Comm comm, int *rank);
int MPI_Comm_size(MPI_Comm comm, int *size);
int MPI_Allreduce(const void *send, void *recv, int count, MPI_Datatype type, MPI_Op op, MPI_Comm comm);
int MPI_Reduce(const void *send, void *recv, int count, MPI_Datatype type, MPI_Op op, int root, MPI_Comm comm);
int MPI_Gather(const void *send, int scount, MPI_Datatype stype, void *recv, int rcount, MPI_Datatype rtype,
               int root, MPI_Comm comm);
int MPI_Scatter(const void *send, int scount, MPI_Datatype stype, void *recv, int rcount, MPI_Datatype rtype,
                int root, MPI_Comm comm);
int MPI_Exscan(const void *send, void *recv, int count, MPI_Datatype type, MPI_Op op, MPI_Comm comm);
int MPI_Allgather(const void *send, int scount, MPI_Datatype stype, void *recv, int rcount, MPI_Datatype rtype,
                  MPI_Comm comm);
int MPI_Bcast(void *buf, int count, MPI_Datatype type, int root, MPI_Comm comm);
int MPI_Barrier(MPI_Comm comm);
int MPI_Abort(MPI_Comm comm, int code);

/* ---- error codes (petscerror.h numbering) and macros ---- */
#define PETSC_SUCCESS 0
#define PETSC_ERR_MEM 55
#define PETSC_ERR_SUP 56
#define PETSC_ERR_SIG 59
#define PETSC_ERR_ARG_WRONG 62
#define PETSC_ERR_ARG_CORRUPT 64
#define PETSC_ERR_ARG_OUTOFRANGE 63
#define PETSC_ERR_ARG_BADPTR 68
#define PETSC_ERR_ARG_NOTSAMETYPE 69
#define PETSC_ERR_ARG_WRONGSTATE 73
#define PETSC_ERR_ARG_INCOMP 75
#define PETSC_ERR_LIB 76
#define PETSC_ERR_PLIB 77
#define PETSC_ERR_FILE_OPEN 65
#define PETSC_ERR_FILE_READ 66
#define PETSC_ERR_FILE_WRITE 67
#define PETSC_ERR_FILE_UNEXPECTED 79
#define PETSC_ERR_CONV_FAILED 91
#define PETSC_ERR_NOT_CONVERGED 91
#define PETSC_ERR_USER 83
#define PETSC_ERR_ARG_NULL 85
#define PETSC_ERR_ARG_UNKNOWN_TYPE 86
#define PETSC_ERR_ARG_UNKNOWN 86
#define PETSC_ERR_ARG_SIZ 60
#define PETSC_ERR_ARG_IDN 61
#define PETSC_ERR_FLOP_COUNT 90
#define PETSC_ERR_POINTER 70
#define PETSC_ERR_GPU 97

/* Records the first error message of a failing call chain (minipetsc_last_error()). */
PetscErrorCode minipetsc_seterr(const char *func, const char *file, int line, PetscErrorCode code,
                                const char *fmt, ...);
const char *minipetsc_last_error(void);
void minipetsc_clear_error(void);

#define SETERRQ(comm, code, ...) return minipetsc_seterr(__func__, __FILE__, __LINE__, (code), __VA_ARGS__)
#define SETERRABORT(comm, code, ...) minipetsc_seterr(__func__, __FILE__, __LINE__, (code), __VA_ARGS__)
#define CHKERRQ(e) do { PetscErrorCode e__ = (e); if (e__) return e__; } while (0)
#define CHKERRMPI(e) CHKERRQ(e)
#define PetscCall(e) do { PetscErrorCode e__ = (e); if (e__) return e__; } while (0)
#define PetscCallMPI(e) PetscCall(e)
#define PetscCheck(cond, comm, code, ...) do { if (!(cond)) SETERRQ(comm, code, __VA_ARGS__); } while (0)
#define PetscFunctionBegin do { } while (0)
#define PetscFunctionBeginUser do { } while (0)
#define PetscFunctionReturn(v) return (v)
#define PetscMin(a, b) (((a) < (b)) ? (a) : (b))
#define PetscMax(a, b) (((a) < (b)) ? (b) : (a))
#define PetscAbsReal(a) fabs(a)
#define PetscAbsScalar(a) fabs(a)
#define PetscSqrtReal(a) sqrt(a)
#define PetscRealPart(a) (a)
#define PetscSqr(a) ((a) * (a))
#define PETSC_MAX_REAL 1.7976931348623157e+308
#define PETSC_MIN_REAL (-PETSC_MAX_REAL)
#define PETSC_MACHINE_EPSILON 2.2204460492503131e-16
#define PETSC_SMALL 1.0e-10
#define PETSC_PI 3.14159265358979323846264338327950288419716939937510582
#define PETSC_MAX_INT INT64_MAX
#define PETSC_MIN_INT INT64_MIN
#define PETSC_DECIDE (-1)
#define PETSC_DETERMINE PETSC_DECIDE
#define PETSC_DEFAULT (-2)
#define PETSC_NULL NULL
#define PETSC_STDOUT stdout
#define PETSC_MAX_PATH_LEN 4096
#define PETSC_VIEWER_STDOUT_SELF ((PetscViewer)0)
#define PETSC_VIEWER_STDOUT_WORLD ((PetscViewer)0)
#define PETSC_EXTERN extern
#define PETSC_INTERN extern
#define PetscUnlikely(c) (c)
#define PetscLikely(c) (c)

/* ---- memory ---- */
PetscErrorCode minipetsc_malloc(size_t bytes, void **p, int zero);
PetscErrorCode minipetsc_realloc(size_t bytes, void **p);
#define PetscMalloc(sz, p) minipetsc_malloc((size_t)(sz), (void **)(p), 0)
#define PetscMalloc1(n, p) minipetsc_malloc((size_t)(n) * sizeof(**(p)), (void **)(p), 0)
#define PetscCalloc(sz, p) minipetsc_malloc((size_t)(sz), (void **)(p), 1)
#define PetscCalloc1(n, p) minipetsc_malloc((size_t)(n) * sizeof(**(p)), (void **)(p), 1)
#define PetscRealloc(sz, p) minipetsc_realloc((size_t)(sz), (void **)(p))
#define PetscFree(p) (free(p), (p) = NULL, PETSC_SUCCESS)
#define PetscMemcpy(a, b, n) (memcpy((a), (b), (n)), PETSC_SUCCESS)
#define PetscArraycpy(a, b, n) (memcpy((a), (b), (size_t)(n) * sizeof(*(a))), PETSC_SUCCESS)
#define PetscMemzero(a, n) (memset((a), 0, (n)), PETSC_SUCCESS)
#define PetscArrayzero(a, n) (memset((a), 0, (size_t)(n) * sizeof(*(a))), PETSC_SUCCESS)
PetscErrorCode PetscSortInt64(PetscInt n, PetscInt64 x[]);
PetscErrorCode PetscSortInt(PetscInt n, PetscInt x[]);
PetscErrorCode PetscStrallocpy(const char s[], char *t[]);
PetscErrorCode PetscStrcmp(const char a[], const char b[], PetscBool *flg);

/* ---- printing, options, timing, logging (quiet) ---- */
PetscErrorCode PetscPrintf(MPI_Comm comm, const char fmt[], ...);
PetscErrorCode PetscSynchronizedPrintf(MPI_Comm comm, const char fmt[], ...);
PetscErrorCode PetscSynchronizedFlush(MPI_Comm comm, FILE *fd);
PetscErrorCode PetscFPrintf(MPI_Comm comm, FILE *fd, const char fmt[], ...);
PetscErrorCode PetscSNPrintf(char *str, size_t len, const char fmt[], ...);
PetscErrorCode PetscInfo(PetscObject obj, const char fmt[], ...);
PetscErrorCode PetscTime(PetscLogDouble *t);
PetscErrorCode PetscLogEventRegister(const char name[], PetscClassId cid, PetscLogEvent *e);
PetscErrorCode PetscLogEventBegin(PetscLogEvent e, PetscObject o1, PetscObject o2, PetscObject o3, PetscObject o4);
PetscErrorCode PetscLogEventEnd(PetscLogEvent e, PetscObject o1, PetscObject o2, PetscObject o3, PetscObject o4);
PetscErrorCode PetscOptionsGetInt(void *opts, const char pre[], const char name[], PetscInt *v, PetscBool *set);
PetscErrorCode PetscOptionsGetReal(void *opts, const char pre[], const char name[], PetscReal *v, PetscBool *set);
PetscErrorCode PetscOptionsGetBool(void *opts, const char pre[], const char name[], PetscBool *v, PetscBool *set);
PetscErrorCode PetscOptionsGetString(void *opts, const char pre[], const char name[], char v[], size_t len,
                                     PetscBool *set);
PetscErrorCode PetscOptionsHasName(void *opts, const char pre[], const char name[], PetscBool *set);
PetscErrorCode PetscOptionsInsertFile(MPI_Comm comm, void *opts, const char file[], PetscBool require);
PetscErrorCode PetscTestFile(const char name[], char mode, PetscBool *flg);
PetscErrorCode PetscBarrier(PetscObject obj);

/* ---- objects ---- */
PetscErrorCode PetscObjectSetName(PetscObject obj, const char name[]);
PetscErrorCode PetscObjectGetName(PetscObject obj, const char *name[]);
PetscErrorCode PetscObjectGetComm(PetscObject obj, MPI_Comm *comm);
MPI_Comm PetscObjectComm(PetscObject obj);
PetscErrorCode PetscObjectStateGet(PetscObject obj, PetscObjectState *state);

/* ---- Vec ---- */
PetscErrorCode VecCreate(MPI_Comm comm, Vec *v);
PetscErrorCode VecCreateSeq(MPI_Comm comm, PetscInt n, Vec *v);
PetscErrorCode VecSetSizes(Vec v, PetscInt n, PetscInt N);
PetscErrorCode VecSetBlockSize(Vec v, PetscInt bs);
PetscErrorCode VecSetFromOptions(Vec v);
PetscErrorCode VecDuplicate(Vec v, Vec *w);
PetscErrorCode VecDestroy(Vec *v);
PetscErrorCode VecCopy(Vec x, Vec y);
PetscErrorCode VecSet(Vec v, PetscScalar a);
PetscErrorCode VecZeroEntries(Vec v);
PetscErrorCode VecGetSize(Vec v, PetscInt *n);
PetscErrorCode VecGetLocalSize(Vec v, PetscInt *n);
PetscErrorCode VecGetBlockSize(Vec v, PetscInt *bs);
PetscErrorCode VecGetDM(Vec v, DM *dm);
PetscErrorCode VecGetArray(Vec v, PetscScalar **a);
PetscErrorCode VecRestoreArray(Vec v, PetscScalar **a);
PetscErrorCode VecGetArrayRead(Vec v, const PetscScalar **a);
PetscErrorCode VecRestoreArrayRead(Vec v, const PetscScalar **a);
PetscErrorCode VecAssemblyBegin(Vec v);
PetscErrorCode VecAssemblyEnd(Vec v);
PetscErrorCode VecSum(Vec v, PetscScalar *s);
PetscErrorCode VecMean(Vec v, PetscScalar *m);
PetscErrorCode VecMax(Vec v, PetscInt *idx, PetscReal *m);
PetscErrorCode VecMin(Vec v, PetscInt *idx, PetscReal *m);
PetscErrorCode VecNorm(Vec v, NormType t, PetscReal *nrm);
PetscErrorCode VecView(Vec v, PetscViewer viewer);
PetscErrorCode VecLoad(Vec v, PetscViewer viewer);
PetscErrorCode VecAXPY(Vec y, PetscScalar a, Vec x);
PetscErrorCode VecScale(Vec v, PetscScalar a);

/* ---- viewers (not supported: the path writes no files through PETSc) ---- */
PetscErrorCode PetscViewerBinaryOpen(MPI_Comm comm, const char name[], PetscFileMode mode, PetscViewer *viewer);
PetscErrorCode PetscViewerDestroy(PetscViewer *viewer);

/* ---- random numbers (seeded rand48 stream; the particle path does not use them) ---- */
PetscErrorCode PetscRandomCreate(MPI_Comm comm, PetscRandom *r);
PetscErrorCode PetscRandomSetType(PetscRandom r, PetscRandomType type);
PetscErrorCode PetscRandomSetInterval(PetscRandom r, PetscScalar lo, PetscScalar hi);
PetscErrorCode PetscRandomSetSeed(PetscRandom r, unsigned long seed);
PetscErrorCode PetscRandomSeed(PetscRandom r);
PetscErrorCode PetscRandomGetValueReal(PetscRandom r, PetscReal *v);
PetscErrorCode PetscRandomGetValue(PetscRandom r, PetscScalar *v);
PetscErrorCode PetscRandomSetFromOptions(PetscRandom r);
PetscErrorCode PetscRandomDestroy(PetscRandom *r);

/* ---- DM / DMDA ---- */
PetscErrorCode DMCreate(MPI_Comm comm, DM *dm);
PetscErrorCode DMSetType(DM dm, DMType type);
PetscErrorCode DMSetDimension(DM dm, PetscInt dim);
PetscErrorCode DMSetFromOptions(DM dm);
PetscErrorCode DMSetUp(DM dm);
PetscErrorCode DMDestroy(DM *dm);
PetscErrorCode DMView(DM dm, PetscViewer viewer);
PetscErrorCode DMDACreate3d(MPI_Comm comm, DMBoundaryType bx, DMBoundaryType by, DMBoundaryType bz,
                            DMDAStencilType st, PetscInt M, PetscInt N, PetscInt P, PetscInt m, PetscInt n,
                            PetscInt p, PetscInt dof, PetscInt s, const PetscInt lx[], const PetscInt ly[],
                            const PetscInt lz[], DM *da);
PetscErrorCode DMDAGetLocalInfo(DM da, DMDALocalInfo *info);
PetscErrorCode DMDAGetInfo(DM da, PetscInt *dim, PetscInt *M, PetscInt *N, PetscInt *P, PetscInt *m, PetscInt *n,
                           PetscInt *p, PetscInt *dof, PetscInt *s, DMBoundaryType *bx, DMBoundaryType *by,
                           DMBoundaryType *bz, DMDAStencilType *st);
PetscErrorCode DMDAGetCorners(DM da, PetscInt *x, PetscInt *y, PetscInt *z, PetscInt *m, PetscInt *n, PetscInt *p);
PetscErrorCode DMDAGetGhostCorners(DM da, PetscInt *x, PetscInt *y, PetscInt *z, PetscInt *m, PetscInt *n,
                                   PetscInt *p);
PetscErrorCode DMDAGetNeighbors(DM da, const PetscMPIInt *ranks[]);
PetscErrorCode DMDASetNumProcs(DM da, PetscInt m, PetscInt n, PetscInt p);
PetscErrorCode DMDAVecGetArray(DM da, Vec v, void *array);
PetscErrorCode DMDAVecRestoreArray(DM da, Vec v, void *array);
PetscErrorCode DMDAVecGetArrayRead(DM da, Vec v, void *array);
PetscErrorCode DMDAVecRestoreArrayRead(DM da, Vec v, void *array);
PetscErrorCode DMDAVecGetArrayDOF(DM da, Vec v, void *array);
PetscErrorCode DMDAVecRestoreArrayDOF(DM da, Vec v, void *array);
PetscErrorCode DMDAVecGetArrayDOFRead(DM da, Vec v, void *array);
PetscErrorCode DMDAVecRestoreArrayDOFRead(DM da, Vec v, void *array);
PetscErrorCode DMGetCoordinateDM(DM dm, DM *cdm);
PetscErrorCode DMGetCoordinates(DM dm, Vec *c);
PetscErrorCode DMGetCoordinatesLocal(DM dm, Vec *c);
PetscErrorCode DMCreateGlobalVector(DM dm, Vec *v);
PetscErrorCode DMCreateLocalVector(DM dm, Vec *v);
PetscErrorCode DMGetLocalVector(DM dm, Vec *v);
PetscErrorCode DMRestoreLocalVector(DM dm, Vec *v);
PetscErrorCode DMGetGlobalVector(DM dm, Vec *v);
PetscErrorCode DMRestoreGlobalVector(DM dm, Vec *v);
PetscErrorCode DMGlobalToLocal(DM dm, Vec g, InsertMode mode, Vec l);
PetscErrorCode DMGlobalToLocalBegin(DM dm, Vec g, InsertMode mode, Vec l);
PetscErrorCode DMGlobalToLocalEnd(DM dm, Vec g, InsertMode mode, Vec l);
PetscErrorCode DMLocalToGlobal(DM dm, Vec l, InsertMode mode, Vec g);
PetscErrorCode DMLocalToGlobalBegin(DM dm, Vec l, InsertMode mode, Vec g);
PetscErrorCode DMLocalToGlobalEnd(DM dm, Vec l, InsertMode mode, Vec g);

/* ---- DMSwarm ---- */
#define DMSwarmPICField_coor "DMSwarmPIC_coor"
#define DMSwarmField_pid "DMSwarm_pid"
#define DMSwarmField_rank "DMSwarm_rank"
PetscErrorCode DMSwarmSetType(DM dm, DMSwarmType type);
PetscErrorCode DMSwarmSetCellDM(DM dm, DM cell);
PetscErrorCode DMSwarmRegisterPetscDatatypeField(DM dm, const char name[], PetscInt bs, PetscDataType type);
PetscErrorCode DMSwarmFinalizeFieldRegister(DM dm);
PetscErrorCode DMSwarmSetLocalSizes(DM dm, PetscInt n, PetscInt buffer);
PetscErrorCode DMSwarmGetLocalSize(DM dm, PetscInt *n);
PetscErrorCode DMSwarmGetSize(DM dm, PetscInt *n);
PetscErrorCode DMSwarmGetField(DM dm, const char name[], PetscInt *bs, PetscDataType *type, void **data);
PetscErrorCode DMSwarmRestoreField(DM dm, const char name[], PetscInt *bs, PetscDataType *type, void **data);
PetscErrorCode DMSwarmAddNPoints(DM dm, PetscInt n);
PetscErrorCode DMSwarmAddPoint(DM dm);
PetscErrorCode DMSwarmRemovePoint(DM dm);
PetscErrorCode DMSwarmRemovePointAtIndex(DM dm, PetscInt idx);
PetscErrorCode DMSwarmMigrate(DM dm, PetscBool remove_sent);
PetscErrorCode DMSwarmCreateGlobalVectorFromField(DM dm, const char name[], Vec *v);
PetscErrorCode DMSwarmDestroyGlobalVectorFromField(DM dm, const char name[], Vec *v);
PetscErrorCode DMSwarmCreateLocalVectorFromField(DM dm, const char name[], Vec *v);
PetscErrorCode DMSwarmDestroyLocalVectorFromField(DM dm, const char name[], Vec *v);
PetscErrorCode DMSwarmVectorDefineField(DM dm, const char name[]);

/* ---- constructors and helpers of this stand-in (not PETSc API) ---- */
/* A one-rank DMDA of M x N x P points with dof components; coordinates (optional) is a Vec of
 * 3 M N P values [P][N][M][3] that DMGetCoordinates(Local) return, with a dof-3 DMDA of the
 * same points as its coordinate DM. */
PetscErrorCode minipetsc_dmda_create(PetscInt M, PetscInt N, PetscInt P, PetscInt dof, DM *da);
PetscErrorCode minipetsc_dm_set_coordinates(DM da, DM cdm, Vec coords);
/* A Vec of n values on dm (dm may be NULL) with block size bs, zeroed. */
PetscErrorCode minipetsc_vec_create(DM dm, PetscInt n, PetscInt bs, Vec *v);
/* The Vec's storage (contiguous, length n). */
PetscScalar *minipetsc_vec_data(Vec v);
PetscInt minipetsc_vec_length(Vec v);
/* Bumps the Vec's state counter (PetscObjectStateGet) after a direct write to its storage. */
void minipetsc_vec_touch(Vec v);
/* Number of DMSwarmGetField views still held (every Get must be matched by a Restore). */
int minipetsc_swarm_fields_held(DM dm);

#ifdef __cplusplus
}
#endif
#endif
