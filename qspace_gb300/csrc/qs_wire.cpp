// Binary wire container of a QSpace ("QSPW"): the MATLAB struct {Q, data,
// info.itags} of the reference (Source/QSpace.hh:3005-3100: QSpace::toMx and
// the mxArray constructor; QSpace.hh:3151-3300) as one flat, position-
// independent buffer that can be sent, stored or memory-mapped and read in
// place.  Abelian QSpaces only: the non-abelian CGR references of info.cgr
// (CRef fields, Source/clebsch_io.cc:1720-1737) have no section.
//
// Layout (little-endian; every section starts on a 64-byte boundary):
//   header   128 bytes (WireHeader below)
//   labels   int32[nblk * rank * qdim], block-major as in qs_qspace_view
//   dims     int64[nblk * rank]
//   offsets  int64[nblk], element offsets into the data section
//   data     double[nelem] (complex: {re, im} pairs, 2 * nelem doubles)
//   itags    "a,b*,c" and a terminating NUL (one NUL when there are none)
// The data section is 64-byte aligned, so a device copy can start from it.
#include <cuda_runtime.h>

#include <cstring>
#include <memory>
#include <string>

#include "qs_objects.h"

namespace {

constexpr uint32_t WIRE_VERSION = 1;
constexpr uint32_t WIRE_ENDIAN = 0x01020304u;  // as the producer stored it
constexpr int64_t WIRE_ALIGN = 64;

struct WireHeader {
  char magic[4];       // "QSPW"
  uint32_t version;    // WIRE_VERSION
  uint32_t flags;      // bit 0: complex data
  int32_t rank, qdim;
  uint32_t endian;     // WIRE_ENDIAN
  int64_t nblk;
  int64_t nelem;       // extent of the data section in elements
  int64_t off_q, off_dims, off_offs, off_data, off_itags;
  int64_t len_itags;   // bytes including the NUL
  int64_t total;       // bytes of the whole container
  int64_t reserved[4];
};
static_assert(sizeof(WireHeader) == 128, "wire header is 128 bytes");

int64_t align_up(int64_t x) { return (x + WIRE_ALIGN - 1) / WIRE_ALIGN * WIRE_ALIGN; }

// Section offsets of a container for the given metadata.
WireHeader layout(const qs::QMeta &m, const std::string &tags) {
  WireHeader h{};
  std::memcpy(h.magic, "QSPW", 4);
  h.version = WIRE_VERSION;
  h.flags = m.cplx ? 1u : 0u;
  h.rank = m.rank;
  h.qdim = m.qdim;
  h.endian = WIRE_ENDIAN;
  h.nblk = m.nblk;
  h.nelem = m.nelem;
  int64_t o = align_up((int64_t)sizeof(WireHeader));
  h.off_q = o;
  o = align_up(o + m.nblk * m.rank * m.qdim * 4);
  h.off_dims = o;
  o = align_up(o + m.nblk * m.rank * 8);
  h.off_offs = o;
  o = align_up(o + m.nblk * 8);
  h.off_data = o;
  o = align_up(o + m.nelem * (m.cplx ? 16 : 8));
  h.off_itags = o;
  h.len_itags = (int64_t)tags.size() + 1;
  h.total = o + h.len_itags;
  return h;
}

// Metadata part of a container (header, labels, dims, offsets, itags); the
// caller fills the data section.
void write_meta(const qs::QMeta &m, const std::string &tags, const WireHeader &h, uint8_t *buf) {
  std::memset(buf, 0, (size_t)h.off_data);  // header, sections and their padding
  std::memcpy(buf, &h, sizeof(h));
  if (!m.q.empty()) std::memcpy(buf + h.off_q, m.q.data(), m.q.size() * 4);
  if (!m.dims.empty()) std::memcpy(buf + h.off_dims, m.dims.data(), m.dims.size() * 8);
  if (!m.offs.empty()) std::memcpy(buf + h.off_offs, m.offs.data(), m.offs.size() * 8);
  const int64_t data_end = h.off_data + m.nelem * (m.cplx ? 16 : 8);
  std::memset(buf + data_end, 0, (size_t)(h.off_itags - data_end));
  std::memcpy(buf + h.off_itags, tags.c_str(), tags.size() + 1);
}

// Checks a container and points a view into it; every length and offset is
// validated before a pointer is formed.
qs_qspace_view read_view(const void *buf, int64_t bytes) {
  using qs::fail;
  if (!buf) fail(QS_ERR_ARG, "wire: null buffer");
  if (bytes < (int64_t)sizeof(WireHeader)) fail(QS_ERR_ARG, "wire: %lld bytes, shorter than the header", (long long)bytes);
  if (reinterpret_cast<uintptr_t>(buf) % 8) fail(QS_ERR_ARG, "wire: buffer not 8-byte aligned");
  WireHeader h;
  std::memcpy(&h, buf, sizeof(h));
  if (std::memcmp(h.magic, "QSPW", 4)) fail(QS_ERR_ARG, "wire: not a QSpace container (bad magic)");
  if (h.endian != WIRE_ENDIAN) fail(QS_ERR_ARG, "wire: container written with another byte order");
  if (h.version != WIRE_VERSION) fail(QS_ERR_UNSUPPORTED, "wire: format version %u (this library reads %u)", h.version, WIRE_VERSION);
  if (h.flags & ~1u) fail(QS_ERR_ARG, "wire: unknown flags 0x%x", h.flags);
  if (h.rank < 0 || h.rank > 8 || h.qdim < 0 || h.qdim > 16 || h.nblk < 0 || h.nblk > (int64_t(1) << 40) ||
      h.nelem < 0 || h.nelem > (int64_t(1) << 50) || h.len_itags < 1)
    fail(QS_ERR_ARG, "wire: header fields out of range");
  if (h.total > bytes) fail(QS_ERR_ARG, "wire: container of %lld bytes in a buffer of %lld", (long long)h.total, (long long)bytes);
  const int64_t es = (h.flags & 1) ? 16 : 8;
  struct Sec { int64_t off, len; } sec[5] = {{h.off_q, h.nblk * h.rank * h.qdim * 4},
                                              {h.off_dims, h.nblk * h.rank * 8},
                                              {h.off_offs, h.nblk * 8},
                                              {h.off_data, h.nelem * es},
                                              {h.off_itags, h.len_itags}};
  int64_t prev_end = (int64_t)sizeof(WireHeader);
  for (const Sec &s : sec) {
    if (s.off % WIRE_ALIGN || s.off < prev_end || s.len < 0 || s.off > h.total || s.len > h.total - s.off)
      fail(QS_ERR_ARG, "wire: section [%lld,+%lld) misplaced", (long long)s.off, (long long)s.len);
    prev_end = s.off + s.len;
  }
  const char *base = static_cast<const char *>(buf);
  if (base[h.off_itags + h.len_itags - 1] != 0) fail(QS_ERR_ARG, "wire: itags not NUL-terminated");
  if ((int64_t)std::strlen(base + h.off_itags) != h.len_itags - 1) fail(QS_ERR_ARG, "wire: NUL inside the itags");
  qs_qspace_view v{};
  v.rank = h.rank;
  v.qdim = h.qdim;
  v.nblk = h.nblk;
  v.q = reinterpret_cast<const int32_t *>(base + h.off_q);
  v.dims = reinterpret_cast<const int64_t *>(base + h.off_dims);
  v.offs = reinterpret_cast<const int64_t *>(base + h.off_offs);
  v.data = reinterpret_cast<const double *>(base + h.off_data);
  v.is_complex = (h.flags & 1) ? 1 : 0;
  v.itags = h.len_itags > 1 ? base + h.off_itags : nullptr;
  // block dims / offsets must stay inside the data section (same checks as
  // every other entry point that takes a view)
  const qs::QMeta m = qs::meta_from_view(&v);
  if (m.nelem > h.nelem) fail(QS_ERR_SHAPE, "wire: blocks reach element %lld of a %lld-element data section", (long long)m.nelem, (long long)h.nelem);
  return v;
}

}  // namespace

using qs::fail;
using qs::QMeta;

qs_status qs_wire_size(const qs_qspace_view *A, int64_t *bytes) {
  QS_API_BEGIN
  if (!bytes) fail(QS_ERR_ARG, "null size pointer");
  const QMeta m = qs::meta_from_view(A);
  *bytes = layout(m, qs::join_itags(m.itags)).total;
  QS_API_END
}

qs_status qs_wire_pack(const qs_qspace_view *A, void *buf, int64_t bytes) {
  QS_API_BEGIN
  const QMeta m = qs::meta_from_view(A);
  const std::string tags = qs::join_itags(m.itags);
  const WireHeader h = layout(m, tags);
  if (!buf) fail(QS_ERR_ARG, "null buffer");
  if (bytes < h.total) fail(QS_ERR_ARG, "wire buffer of %lld bytes, %lld needed", (long long)bytes, (long long)h.total);
  uint8_t *b = static_cast<uint8_t *>(buf);
  write_meta(m, tags, h, b);
  if (m.nelem) std::memcpy(b + h.off_data, A->data, (size_t)m.nelem * (m.cplx ? 16 : 8));
  QS_API_END
}

qs_status qs_wire_view(const void *buf, int64_t bytes, qs_qspace_view *A) {
  QS_API_BEGIN
  if (!A) fail(QS_ERR_ARG, "null view");
  *A = read_view(buf, bytes);
  QS_API_END
}

qs_status qs_tensor_from_wire(qs_ctx *ctx, const void *buf, int64_t bytes, qs_tensor **out) {
  QS_API_BEGIN
  if (!ctx || !out) fail(QS_ERR_ARG, "null argument");
  const qs_qspace_view v = read_view(buf, bytes);
  return qs_tensor_upload(ctx, &v, out);
  QS_API_END
}

qs_status qs_tensor_wire_size(const qs_tensor *T, int64_t *bytes) {
  QS_API_BEGIN
  if (!T || !bytes) fail(QS_ERR_ARG, "null argument");
  *bytes = layout(T->meta, qs::join_itags(T->meta.itags)).total;
  QS_API_END
}

qs_status qs_tensor_to_wire(qs_ctx *ctx, const qs_tensor *T, void *buf, int64_t bytes) {
  QS_API_BEGIN
  if (!ctx || !T || !buf) fail(QS_ERR_ARG, "null argument");
  const QMeta &m = T->meta;
  const std::string tags = qs::join_itags(m.itags);
  const WireHeader h = layout(m, tags);
  if (bytes < h.total) fail(QS_ERR_ARG, "wire buffer of %lld bytes, %lld needed", (long long)bytes, (long long)h.total);
  uint8_t *b = static_cast<uint8_t *>(buf);
  write_meta(m, tags, h, b);
  // the device arena goes straight into the data section (one copy)
  qs::Ctx *c = &ctx->c;
  QS_CUDA(cudaSetDevice(c->device));
  if (m.nelem)
    QS_CUDA(cudaMemcpyAsync(b + h.off_data, T->d, (size_t)m.nelem * (m.cplx ? 16 : 8), cudaMemcpyDeviceToHost,
                            c->stream));
  QS_CUDA(cudaStreamSynchronize(c->stream));
  QS_API_END
}
