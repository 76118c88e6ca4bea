// petsc_io.cpp -- PETSc binary Vec files, so states move between this library
// and the reference's drivers. The reference writes its states with VecView on
// a binary viewer (write_vector_to_binary, code/src/util/io_util.cpp:4-14).
//
// Format (PETSc's documented binary layout for a Vec, default 32-bit
// PetscInt): big-endian int32 VEC_FILE_CLASSID = 1211214, big-endian int32
// number of entries, then the entries as big-endian IEEE doubles. A
// single-rank DMDA vector is written in its natural ordering, which is the
// AoS order dofs*(i + nx*j) + comp used at this library's boundary.
#include <cstdint>
#include <cstdio>
#include <cstring>

#include "../../include/sbpgpu.h"

namespace {

constexpr int32_t kVecClassId = 1211214;

void put_be32(unsigned char* p, uint32_t v) {
  p[0] = (unsigned char)(v >> 24);
  p[1] = (unsigned char)(v >> 16);
  p[2] = (unsigned char)(v >> 8);
  p[3] = (unsigned char)v;
}

uint32_t get_be32(const unsigned char* p) {
  return ((uint32_t)p[0] << 24) | ((uint32_t)p[1] << 16) | ((uint32_t)p[2] << 8) | (uint32_t)p[3];
}

void put_be64(unsigned char* p, uint64_t v) {
  for (int k = 0; k < 8; k++) p[k] = (unsigned char)(v >> (56 - 8 * k));
}

uint64_t get_be64(const unsigned char* p) {
  uint64_t v = 0;
  for (int k = 0; k < 8; k++) v = (v << 8) | p[k];
  return v;
}

}  // namespace

extern "C" int sbp_write_petsc_vec(const char* path, const double* v, long long n) {
  if (!path || (!v && n > 0) || n < 0 || n > 0x7fffffffLL) return SBP_ERR_INVALID;
  FILE* f = std::fopen(path, "wb");
  if (!f) return SBP_ERR_INVALID;
  unsigned char head[8];
  put_be32(head, (uint32_t)kVecClassId);
  put_be32(head + 4, (uint32_t)n);
  bool ok = std::fwrite(head, 1, 8, f) == 8;
  unsigned char buf[8 * 1024];
  for (long long i = 0; ok && i < n;) {
    const long long m = (n - i) < 1024 ? (n - i) : 1024;
    for (long long k = 0; k < m; k++) {
      uint64_t bits;
      std::memcpy(&bits, v + i + k, 8);
      put_be64(buf + 8 * k, bits);
    }
    ok = std::fwrite(buf, 8, (size_t)m, f) == (size_t)m;
    i += m;
  }
  ok = (std::fclose(f) == 0) && ok;
  return ok ? SBP_OK : SBP_ERR_INVALID;
}

extern "C" int sbp_read_petsc_vec(const char* path, double* v, long long capacity, long long* n) {
  if (!path || !n) return SBP_ERR_INVALID;
  FILE* f = std::fopen(path, "rb");
  if (!f) return SBP_ERR_INVALID;
  unsigned char head[8];
  if (std::fread(head, 1, 8, f) != 8 || (int32_t)get_be32(head) != kVecClassId) {
    std::fclose(f);
    return SBP_ERR_INVALID;
  }
  const long long len = (long long)(int32_t)get_be32(head + 4);
  *n = len;
  if (len < 0 || !v || len > capacity) {
    std::fclose(f);
    return (len >= 0 && !v) ? SBP_OK : SBP_ERR_INVALID;  // v == NULL: query the length only
  }
  unsigned char buf[8 * 1024];
  bool ok = true;
  for (long long i = 0; ok && i < len;) {
    const long long m = (len - i) < 1024 ? (len - i) : 1024;
    ok = std::fread(buf, 8, (size_t)m, f) == (size_t)m;
    for (long long k = 0; ok && k < m; k++) {
      const uint64_t bits = get_be64(buf + 8 * k);
      std::memcpy(v + i + k, &bits, 8);
    }
    i += m;
  }
  std::fclose(f);
  return ok ? SBP_OK : SBP_ERR_INVALID;
}
