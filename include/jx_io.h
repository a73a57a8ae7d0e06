/*
 * jx host I/O: the reference's binary CSR file format, version 2.
 *
 * Reference: readMtxToCSR.hpp:44-64 (CSRFileHeader), readMtxToCSR.cpp:285-395 (CSRToFile,
 * CSRFileReader, FileToCSR).  Layout, little-endian:
 *   int64 version (= 2), int64 numVerts, int64 numEdges, 8-byte flags word with
 *   bit 0 isWeighted, 1 isZeroIndexed, 2 isDirected, 3 hasReverseEdges, 4 isVertexT64,
 *   5 isEdgeT64, 6 isWeightT64, bits 7..63 zero;
 *   then offsets[numVerts + 1] (int64 if isEdgeT64 else int32), indices[numEdges] (int64 if
 *   isVertexT64 else int32), and, if isWeighted, edge weights[numEdges] (double if
 *   isWeightT64 else float).
 * The reference's writer sets isWeightT64 from is_same<WT, int64_t> (readMtxToCSR.cpp:293),
 * so its files with double weights carry isWeightT64 = 0; jx writes the flag from the real
 * weight type (here always float, flag 0), which agrees with the reference for float weights.
 *
 * Plain C, host memory, status codes (0 = ok).
 */
#ifndef JX_IO_H
#define JX_IO_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define JX_CSR_FILE_VERSION 2
#define JX_CSRF_WEIGHTED (1u << 0)
#define JX_CSRF_ZERO_INDEXED (1u << 1)
#define JX_CSRF_DIRECTED (1u << 2)
#define JX_CSRF_REVERSE_EDGES (1u << 3)
#define JX_CSRF_VERTEX_T64 (1u << 4)
#define JX_CSRF_EDGE_T64 (1u << 5)
#define JX_CSRF_WEIGHT_T64 (1u << 6)

enum {
  JX_IO_OK = 0,
  JX_IO_OPEN = 1,     /* cannot open the file */
  JX_IO_SHORT = 2,    /* file shorter than its header says */
  JX_IO_VERSION = 3,  /* not a version-2 CSR file */
  JX_IO_RANGE = 4,    /* a value does not fit int32 (64-bit file read into int32 arrays) */
  JX_IO_INVALID = 5,  /* bad argument */
  JX_IO_WRITE = 6     /* write failed */
};

/* Header of a CSR file. */
int jxio_csr_read_header(const char *path, int64_t *num_verts, int64_t *num_edges, uint64_t *flags);

/* Read a CSR file into caller arrays: offsets int32[num_verts + 1], indices int32[num_edges],
 * edge_weights float[num_edges] (may be NULL; filled only when the file is weighted).  64-bit
 * indices and double weights in the file are converted (indices must fit int32). */
int jxio_csr_read(const char *path, int32_t *offsets, int32_t *indices, float *edge_weights);

/* Write an int32 / float CSR (edge_weights may be NULL); `flags` supplies the
 * isZeroIndexed / isDirected / hasReverseEdges bits, the type and weighted bits are set here. */
int jxio_csr_write(const char *path, int64_t num_verts, int64_t num_edges, const int32_t *offsets,
                   const int32_t *indices, const float *edge_weights, uint64_t flags);

#ifdef __cplusplus
}
#endif

#endif /* JX_IO_H */
