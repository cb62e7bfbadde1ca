/*
 * Single-rank MPI stand-in used only to compile the reference DistPCA sources
 * as a CPU oracle (test infrastructure, never part of the product).
 *
 * Collectives degenerate to copies, MPI-IO becomes pread(2) on a plain file
 * descriptor, and non-blocking reads complete before they return, so
 * MPI_Wait has nothing left to do.  Only the calls the reference makes are
 * provided (distpca.cpp, methods.cpp).
 */
#ifndef DPCA_ORACLE_SHIM_MPI_H
#define DPCA_ORACLE_SHIM_MPI_H

#include <fcntl.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef int MPI_Info;
typedef int MPI_Request;
typedef struct { int fd; } MPI_File;
typedef struct { int count; } MPI_Status;

#define MPI_COMM_WORLD 0
#define MPI_SUCCESS 0
#define MPI_ERR_FILE 27
#define MPI_INFO_NULL 0
#define MPI_MODE_RDONLY 2
#define MPI_MAX_ERROR_STRING 256
#define MPI_DOUBLE 1
#define MPI_UNSIGNED_CHAR 2
#define MPI_SUM 1
#define MPI_REQUEST_NULL 0
#define MPI_STATUS_IGNORE ((MPI_Status *)0)

static inline int dpca_shim_type_size(MPI_Datatype t) { return t == MPI_DOUBLE ? 8 : 1; }

static inline int MPI_Init(int *, char ***) { return MPI_SUCCESS; }
static inline int MPI_Finalize(void) { return MPI_SUCCESS; }
static inline int MPI_Comm_rank(MPI_Comm, int *r) { *r = 0; return MPI_SUCCESS; }
static inline int MPI_Comm_size(MPI_Comm, int *s) { *s = 1; return MPI_SUCCESS; }
static inline int MPI_Barrier(MPI_Comm) { return MPI_SUCCESS; }
static inline int MPI_Abort(MPI_Comm, int code) { exit(code); return code; }

static inline int MPI_Allreduce(const void *in, void *out, int count, MPI_Datatype t, MPI_Op, MPI_Comm) {
    if (in != out) memmove(out, in, (size_t)count * (size_t)dpca_shim_type_size(t));
    return MPI_SUCCESS;
}

static inline int MPI_Error_string(int code, char *s, int *len) {
    *len = snprintf(s, MPI_MAX_ERROR_STRING, "shim MPI error %d", code);
    return MPI_SUCCESS;
}

static inline int MPI_File_open(MPI_Comm, const char *path, int, MPI_Info, MPI_File *fh) {
    fh->fd = open(path, O_RDONLY);
    return fh->fd < 0 ? MPI_ERR_FILE : MPI_SUCCESS;
}

static inline int MPI_File_close(MPI_File *fh) {
    if (fh->fd >= 0) close(fh->fd);
    fh->fd = -1;
    return MPI_SUCCESS;
}

/* Positional read of count elements; loops over short reads. */
static inline int MPI_File_read_at(MPI_File fh, long long off, void *buf, int count, MPI_Datatype t, MPI_Status *) {
    size_t want = (size_t)count * (size_t)dpca_shim_type_size(t);
    char *p = (char *)buf;
    while (want > 0) {
        ssize_t got = pread(fh.fd, p, want, (off_t)off);
        if (got <= 0) return MPI_ERR_FILE;
        p += got;
        off += got;
        want -= (size_t)got;
    }
    return MPI_SUCCESS;
}

static inline int MPI_File_iread_at(MPI_File fh, long long off, void *buf, int count, MPI_Datatype t, MPI_Request *req) {
    *req = MPI_REQUEST_NULL;
    return MPI_File_read_at(fh, off, buf, count, t, 0);
}

static inline int MPI_Wait(MPI_Request *, MPI_Status *) { return MPI_SUCCESS; }

#endif
