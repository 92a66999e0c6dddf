// Sparse brick / voxel set files in the reference's binary layout
// (sdfScene/sdf_scene.cpp:121-175): an SBS file is the 16-byte header, the
// node count (u32), the 16-byte nodes, the value count (u32) and the 32-bit
// values; an SVS file is the node count and the 16-byte nodes.  Host byte
// order, as the reference writes it.  Loading checks every count against the
// file size, so a truncated or foreign file is rejected instead of read past.
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "lrt_internal.h"

namespace {

struct File {
  FILE *f = nullptr;
  explicit File(const char *path, const char *mode) { f = std::fopen(path, mode); }
  ~File() {
    if (f) std::fclose(f);
  }
};

bool file_size(FILE *f, uint64_t &n) {
  if (std::fseek(f, 0, SEEK_END) != 0) return false;
  const long e = std::ftell(f);
  if (e < 0 || std::fseek(f, 0, SEEK_SET) != 0) return false;
  n = uint64_t(e);
  return true;
}

bool read_exact(FILE *f, void *p, size_t n) { return n == 0 || std::fread(p, 1, n, f) == n; }
bool write_exact(FILE *f, const void *p, size_t n) { return n == 0 || std::fwrite(p, 1, n, f) == n; }

}  // namespace

// save_sdf_SBS, sdfScene/sdf_scene.cpp:148-158
extern "C" lrt_status lrt_sbs_save(const char *path, const lrt_sbs_header *hdr, const lrt_sbs_node *nodes,
                                   uint32_t n_nodes, const uint32_t *values, uint32_t n_values) {
  if (!path || !hdr || (n_nodes && !nodes) || (n_values && !values)) return LRT_ERR_INVALID;
  File fl(path, "wb");
  if (!fl.f) return LRT_ERR_INVALID;
  const bool ok = write_exact(fl.f, hdr, sizeof(*hdr)) && write_exact(fl.f, &n_nodes, 4) &&
                  write_exact(fl.f, nodes, size_t(n_nodes) * sizeof(lrt_sbs_node)) && write_exact(fl.f, &n_values, 4) &&
                  write_exact(fl.f, values, size_t(n_values) * 4) && std::fflush(fl.f) == 0;
  return ok ? LRT_OK : LRT_ERR_INVALID;
}

// load_sdf_SBS, sdfScene/sdf_scene.cpp:160-173
extern "C" lrt_status lrt_sbs_load(const char *path, lrt_sbs **out) {
  if (!path || !out) return LRT_ERR_INVALID;
  File fl(path, "rb");
  uint64_t size = 0;
  if (!fl.f || !file_size(fl.f, size)) return LRT_ERR_INVALID;
  lrt_sbs_header hdr;
  uint32_t n = 0, nv = 0;
  if (size < sizeof(hdr) + 8 || !read_exact(fl.f, &hdr, sizeof(hdr)) || !read_exact(fl.f, &n, 4)) return LRT_ERR_INVALID;
  const uint64_t after_nodes = sizeof(hdr) + 4 + uint64_t(n) * sizeof(lrt_sbs_node);
  if (after_nodes + 4 > size) return LRT_ERR_INVALID;
  lrt_sbs *r = new (std::nothrow) lrt_sbs();
  if (!r) return LRT_ERR_OOM;
  r->d.hdr = hdr;
  bool ok = true;
  try {
    r->d.nodes.resize(n);
    ok = read_exact(fl.f, r->d.nodes.data(), size_t(n) * sizeof(lrt_sbs_node)) && read_exact(fl.f, &nv, 4) &&
         after_nodes + 4 + uint64_t(nv) * 4 <= size;
    if (ok) {
      r->d.values.resize(nv);
      ok = read_exact(fl.f, r->d.values.data(), size_t(nv) * 4);
    }
  } catch (const std::bad_alloc &) {
    delete r;
    return LRT_ERR_OOM;
  }
  if (!ok) {
    delete r;
    return LRT_ERR_INVALID;
  }
  *out = r;
  return LRT_OK;
}

// save_sdf_SVS / load_sdf_SVS, sdfScene/sdf_scene.cpp:121-137
extern "C" lrt_status lrt_svs_save(const char *path, const lrt_svs_node *nodes, uint32_t n_nodes) {
  if (!path || (n_nodes && !nodes)) return LRT_ERR_INVALID;
  File fl(path, "wb");
  if (!fl.f) return LRT_ERR_INVALID;
  const bool ok = write_exact(fl.f, &n_nodes, 4) && write_exact(fl.f, nodes, size_t(n_nodes) * sizeof(lrt_svs_node)) &&
                  std::fflush(fl.f) == 0;
  return ok ? LRT_OK : LRT_ERR_INVALID;
}

extern "C" lrt_status lrt_svs_load(const char *path, lrt_svs **out) {
  if (!path || !out) return LRT_ERR_INVALID;
  File fl(path, "rb");
  uint64_t size = 0;
  uint32_t n = 0;
  if (!fl.f || !file_size(fl.f, size) || size < 4 || !read_exact(fl.f, &n, 4)) return LRT_ERR_INVALID;
  if (4 + uint64_t(n) * sizeof(lrt_svs_node) > size) return LRT_ERR_INVALID;
  lrt_svs *r = new (std::nothrow) lrt_svs();
  if (!r) return LRT_ERR_OOM;
  try {
    r->nodes.resize(n);
  } catch (const std::bad_alloc &) {
    delete r;
    return LRT_ERR_OOM;
  }
  if (!read_exact(fl.f, r->nodes.data(), size_t(n) * sizeof(lrt_svs_node))) {
    delete r;
    return LRT_ERR_INVALID;
  }
  *out = r;
  return LRT_OK;
}
