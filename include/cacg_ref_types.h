/*
 * cacg_ref_types.h -- the reference's ABI structs, byte-for-byte.
 *
 * csrType_local and denseType are passed BY VALUE to the drop-in entry points
 * cbcg_v1 / bcbcg_v1, exactly as sclc/cacg declares them in src/DataTypes.h:22-61.
 * This header deliberately uses the reference's include guard (DATATYPES_H):
 * a driver that already includes the reference's DataTypes.h gets the same
 * definitions and this file becomes a no-op, and vice versa.
 */
#ifndef DATATYPES_H
#define DATATYPES_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    long num_rows;
    long num_cols;
    long nnz;
} matInfo;

/* local block of rows of a CSR matrix (src/DataTypes.h:22-41):
 * row_start[num_rows+1] offsets, col_idx[nnz] GLOBAL column indices,
 * csrdata[nnz] values, start = global index of the first local row. */
typedef struct {
    long num_rows, num_cols, nnz;
    long start;
    long *row_start;
    long *col_idx;
    double *csrdata;
} csrType_local;

typedef struct {
    long *rowIdx;
    long *colIdx;
    double *coodata;
} cooType;

/* dense block, row-major: element (i, c) at data[i * local_num_col + c]
 * (src/DataTypes.h:50-59). */
typedef struct {
    long local_num_row;
    long local_num_col;
    long global_num_row;
    long global_num_col;
    long start_idx;
    double *data;
} denseType;

#ifdef __cplusplus
}
#endif

#endif /* DATATYPES_H */
