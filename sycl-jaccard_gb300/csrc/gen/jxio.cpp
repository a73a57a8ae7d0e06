// Binary CSR files, version 2 (the reference's format): see include/jx_io.h.
#include "../../../include/jx_io.h"

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <limits>
#include <memory>
#include <vector>

namespace {

struct Header {
  int64_t version, nv, ne;
  uint64_t flags;
};
static_assert(sizeof(Header) == 32, "CSR file header is 32 bytes");

struct File {
  FILE *f = nullptr;
  explicit File(const char *path, const char *mode) : f(std::fopen(path, mode)) {}
  ~File() {
    if (f) std::fclose(f);
  }
};

int read_header(FILE *f, Header *h) {
  if (std::fread(h, sizeof(Header), 1, f) != 1) return JX_IO_SHORT;
  if (h->version != JX_CSR_FILE_VERSION || h->nv < 0 || h->ne < 0) return JX_IO_VERSION;
  return JX_IO_OK;
}

// Read n values of the file's type (64-bit when wide) into int32 `out`, range-checked.
int read_ints(FILE *f, int64_t n, bool wide, int32_t *out) {
  if (!wide) return std::fread(out, sizeof(int32_t), (size_t)n, f) == (size_t)n ? JX_IO_OK : JX_IO_SHORT;
  const int64_t chunk = 1 << 20;
  std::vector<int64_t> buf((size_t)std::min<int64_t>(n, chunk));
  for (int64_t done = 0; done < n;) {
    const int64_t k = std::min<int64_t>(chunk, n - done);
    if (std::fread(buf.data(), sizeof(int64_t), (size_t)k, f) != (size_t)k) return JX_IO_SHORT;
    for (int64_t i = 0; i < k; ++i) {
      if (buf[i] < std::numeric_limits<int32_t>::min() || buf[i] > std::numeric_limits<int32_t>::max())
        return JX_IO_RANGE;
      out[done + i] = (int32_t)buf[i];
    }
    done += k;
  }
  return JX_IO_OK;
}

int read_floats(FILE *f, int64_t n, bool wide, float *out) {
  if (!wide) return std::fread(out, sizeof(float), (size_t)n, f) == (size_t)n ? JX_IO_OK : JX_IO_SHORT;
  const int64_t chunk = 1 << 20;
  std::vector<double> buf((size_t)std::min<int64_t>(n, chunk));
  for (int64_t done = 0; done < n;) {
    const int64_t k = std::min<int64_t>(chunk, n - done);
    if (std::fread(buf.data(), sizeof(double), (size_t)k, f) != (size_t)k) return JX_IO_SHORT;
    for (int64_t i = 0; i < k; ++i) out[done + i] = (float)buf[i];
    done += k;
  }
  return JX_IO_OK;
}

} // namespace

extern "C" {

int jxio_csr_read_header(const char *path, int64_t *num_verts, int64_t *num_edges, uint64_t *flags) {
  if (!path) return JX_IO_INVALID;
  File f(path, "rb");
  if (!f.f) return JX_IO_OPEN;
  Header h;
  const int st = read_header(f.f, &h);
  if (st != JX_IO_OK) return st;
  if (num_verts) *num_verts = h.nv;
  if (num_edges) *num_edges = h.ne;
  if (flags) *flags = h.flags;
  return JX_IO_OK;
}

int jxio_csr_read(const char *path, int32_t *offsets, int32_t *indices, float *edge_weights) {
  if (!path || !offsets || !indices) return JX_IO_INVALID;
  File f(path, "rb");
  if (!f.f) return JX_IO_OPEN;
  Header h;
  int st = read_header(f.f, &h);
  if (st != JX_IO_OK) return st;
  // offsets have the edge type, indices the vertex type (readMtxToCSR.cpp:346-353)
  if ((st = read_ints(f.f, h.nv + 1, h.flags & JX_CSRF_EDGE_T64, offsets)) != JX_IO_OK) return st;
  if ((st = read_ints(f.f, h.ne, h.flags & JX_CSRF_VERTEX_T64, indices)) != JX_IO_OK) return st;
  if ((h.flags & JX_CSRF_WEIGHTED) && edge_weights)
    if ((st = read_floats(f.f, h.ne, h.flags & JX_CSRF_WEIGHT_T64, edge_weights)) != JX_IO_OK) return st;
  return JX_IO_OK;
}

int jxio_csr_write(const char *path, int64_t num_verts, int64_t num_edges, const int32_t *offsets,
                   const int32_t *indices, const float *edge_weights, uint64_t flags) {
  if (!path || num_verts < 0 || num_edges < 0 || !offsets || (num_edges > 0 && !indices)) return JX_IO_INVALID;
  File f(path, "wb");
  if (!f.f) return JX_IO_OPEN;
  Header h{JX_CSR_FILE_VERSION, num_verts, num_edges,
           (flags & (JX_CSRF_ZERO_INDEXED | JX_CSRF_DIRECTED | JX_CSRF_REVERSE_EDGES)) |
               (edge_weights ? JX_CSRF_WEIGHTED : 0u)};
  if (std::fwrite(&h, sizeof h, 1, f.f) != 1) return JX_IO_WRITE;
  if (std::fwrite(offsets, sizeof(int32_t), (size_t)num_verts + 1, f.f) != (size_t)num_verts + 1) return JX_IO_WRITE;
  if (std::fwrite(indices, sizeof(int32_t), (size_t)num_edges, f.f) != (size_t)num_edges) return JX_IO_WRITE;
  if (edge_weights && std::fwrite(edge_weights, sizeof(float), (size_t)num_edges, f.f) != (size_t)num_edges)
    return JX_IO_WRITE;
  return JX_IO_OK;
}

} // extern "C"
