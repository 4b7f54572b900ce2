// Particle output as legacy-VTK polydata, the format of the reference
// driver's writeTovtk (src/main.cpp:127-164): POINTS (X), one VERTICES
// cell per particle, then POINT_DATA with the vectors alpha and velocity
// and the scalar radius.  Host code only.
//
// ASCII mode writes the reference's file byte for byte: every number in
// std::ostream's default format (printf "%g", six significant digits).
// BINARY mode writes the same dataset with full FP64 values as legacy VTK
// binary data (big-endian doubles, 32-bit vertex connectivity).
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <vector>

#include "vfmm.h"

namespace {

struct File {
  FILE *f = nullptr;
  ~File()
  {
    if (f)
      fclose(f);
  }
};

bool host_is_little_endian()
{
  const uint32_t one = 1;
  unsigned char  b;
  memcpy(&b, &one, 1);
  return b == 1;
}

// append v as 8 big-endian bytes
void put_be64(std::vector<unsigned char> &out, double v, bool swap)
{
  unsigned char b[8];
  memcpy(b, &v, 8);
  if (swap)
    for (int i = 0; i < 4; i++) {
      const unsigned char t = b[i];
      b[i]                  = b[7 - i];
      b[7 - i]              = t;
    }
  out.insert(out.end(), b, b + 8);
}

void put_be32(std::vector<unsigned char> &out, int32_t v)
{
  const uint32_t u = (uint32_t)v;
  const unsigned char b[4] = {(unsigned char)(u >> 24), (unsigned char)(u >> 16), (unsigned char)(u >> 8), (unsigned char)u};
  out.insert(out.end(), b, b + 4);
}

bool write_all(FILE *f, const void *p, size_t bytes) { return bytes == 0 || fwrite(p, 1, bytes, f) == bytes; }

bool write_text(FILE *f, std::vector<char> &buf, const char *fmt, ...) __attribute__((format(printf, 3, 4)));
bool write_text(FILE *f, std::vector<char> &buf, const char *fmt, ...)
{
  char    line[256];
  va_list ap;
  va_start(ap, fmt);
  const int k = vsnprintf(line, sizeof line, fmt, ap);
  va_end(ap);
  if (k < 0 || k >= (int)sizeof line)
    return false;
  buf.insert(buf.end(), line, line + k);
  if (buf.size() >= (1u << 20)) {
    if (!write_all(f, buf.data(), buf.size()))
      return false;
    buf.clear();
  }
  return true;
}

int write_ascii(FILE *f, const vfmm_body *b, size_t n)
{
  std::vector<char> buf;
  buf.reserve((1u << 20) + 256);
  bool ok = write_text(f, buf, "# vtk DataFile Version 3.0\nvtk output\nASCII\nDATASET POLYDATA\nPOINTS %zu double\n", n);
  for (size_t i = 0; ok && i < n; i++)
    ok = write_text(f, buf, "%g %g %g\n", b[i].X[0], b[i].X[1], b[i].X[2]);
  ok = ok && write_text(f, buf, "VERTICES %zu %zu\n", n, 2 * n);
  for (size_t i = 0; ok && i < n; i++)
    ok = write_text(f, buf, "1 %zu\n", i);
  ok = ok && write_text(f, buf, "POINT_DATA %zu\nVECTORS alpha double\n", n);
  for (size_t i = 0; ok && i < n; i++)
    ok = write_text(f, buf, "%g %g %g\n", b[i].alpha[0], b[i].alpha[1], b[i].alpha[2]);
  ok = ok && write_text(f, buf, "VECTORS velocity double\n");
  for (size_t i = 0; ok && i < n; i++)
    ok = write_text(f, buf, "%g %g %g\n", b[i].velocity[0], b[i].velocity[1], b[i].velocity[2]);
  ok = ok && write_text(f, buf, "SCALARS radius double\nLOOKUP_TABLE default\n");
  for (size_t i = 0; ok && i < n; i++)
    ok = write_text(f, buf, "%g\n", b[i].radius);
  ok = ok && write_all(f, buf.data(), buf.size());
  return ok ? VFMM_OK : VFMM_ERR_INVALID;
}

int write_binary(FILE *f, const vfmm_body *b, size_t n)
{
  const bool                 swap = host_is_little_endian();
  std::vector<unsigned char> out;
  auto flush = [&]() { return write_all(f, out.data(), out.size()) && (out.clear(), true); };
  auto text  = [&](const char *s) { return write_all(f, s, strlen(s)); };
  char head[160];
  snprintf(head, sizeof head, "# vtk DataFile Version 3.0\nvtk output\nBINARY\nDATASET POLYDATA\nPOINTS %zu double\n", n);
  bool ok = text(head);
  out.reserve(24 * n + 16);
  for (size_t i = 0; i < n; i++)
    for (int d = 0; d < 3; d++)
      put_be64(out, b[i].X[d], swap);
  snprintf(head, sizeof head, "\nVERTICES %zu %zu\n", n, 2 * n);
  ok = ok && flush() && text(head);
  for (size_t i = 0; i < n; i++) {
    put_be32(out, 1);
    put_be32(out, (int32_t)i);
  }
  snprintf(head, sizeof head, "\nPOINT_DATA %zu\nVECTORS alpha double\n", n);
  ok = ok && flush() && text(head);
  for (size_t i = 0; i < n; i++)
    for (int d = 0; d < 3; d++)
      put_be64(out, b[i].alpha[d], swap);
  ok = ok && flush() && text("\nVECTORS velocity double\n");
  for (size_t i = 0; i < n; i++)
    for (int d = 0; d < 3; d++)
      put_be64(out, b[i].velocity[d], swap);
  ok = ok && flush() && text("\nSCALARS radius double\nLOOKUP_TABLE default\n");
  for (size_t i = 0; i < n; i++)
    put_be64(out, b[i].radius, swap);
  ok = ok && flush() && text("\n");
  return ok ? VFMM_OK : VFMM_ERR_INVALID;
}

} // namespace

extern "C" int vfmm_write_vtk(const vfmm_body *bodies, size_t n, const char *path, int binary)
{
  if (!path || (n > 0 && !bodies))
    return VFMM_ERR_INVALID;
  if (binary && n > (size_t)0x7fffffff) // vertex indices are 32-bit in legacy VTK binary data
    return VFMM_ERR_INVALID;
  File f;
  f.f = fopen(path, "wb");
  if (!f.f)
    return VFMM_ERR_INVALID;
  const int rc = binary ? write_binary(f.f, bodies, n) : write_ascii(f.f, bodies, n);
  if (fclose(f.f) != 0) {
    f.f = nullptr;
    return VFMM_ERR_INVALID;
  }
  f.f = nullptr;
  return rc;
}
