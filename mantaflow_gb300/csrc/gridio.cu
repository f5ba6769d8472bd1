// Grid files written straight from the device mirror: Grid<T>::save
// (grid.cpp:135-156) for the .uni, .raw and .npz formats of
// fileio/iogrids.cpp.
//
//  * .uni (writeGridUni, iogrids.cpp:386-432): the 4-byte id "MNT3", the
//    UniHeader (dimensions, grid type flags, element type 0 int / 1 real /
//    2 vec3, bytes per element, a 252-byte info string, dimT, a millisecond
//    timestamp) and the cells in the reference layout (Vec3 interleaved),
//    in one gzip stream.
//  * .raw (writeGridRaw, :255-271): the cells alone, in one gzip stream.
//  * .npz (writeGridNumpy, :836-884): an uncompressed zip holding arr_0.npy
//    with shape (nz, ny, nx, 1 or 3) -- what cnpy::npz_save writes.
//
// The gzip streams use stored (uncompressed) deflate blocks: any gzip reader
// (zlib's gzread, which the reference's readers use, Python's gzip) reads
// them, and the library needs no compression library.  The CRC-32 is the
// IEEE 802.3 polynomial (reflected 0xEDB88320), as gzip and zip specify.
#include <cuda_runtime.h>

#include <chrono>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/mantagpu.h"
#include "mg_batch.h"

using namespace mgpu;

namespace {

uint32_t g_crcTable[256];
bool g_crcReady = false;

void crc_init() {
  if (g_crcReady) return;
  for (uint32_t n = 0; n < 256; n++) {
    uint32_t c = n;
    for (int k = 0; k < 8; k++) c = (c & 1u) ? 0xEDB88320u ^ (c >> 1) : c >> 1;
    g_crcTable[n] = c;
  }
  g_crcReady = true;
}

uint32_t crc_update(uint32_t crc, const unsigned char* p, size_t n) {
  uint32_t c = crc ^ 0xFFFFFFFFu;
  for (size_t i = 0; i < n; i++) c = g_crcTable[(c ^ p[i]) & 0xFFu] ^ (c >> 8);
  return c ^ 0xFFFFFFFFu;
}

void put16(std::vector<unsigned char>& b, uint32_t v) {
  b.push_back((unsigned char)(v & 0xFF));
  b.push_back((unsigned char)((v >> 8) & 0xFF));
}
void put32(std::vector<unsigned char>& b, uint32_t v) {
  put16(b, v & 0xFFFF);
  put16(b, v >> 16);
}

// one gzip member (RFC 1952) holding `parts` concatenated, in stored
// deflate blocks (RFC 1951, BTYPE 00) of at most 65535 bytes
bool write_gzip(FILE* f, const std::vector<std::pair<const void*, size_t>>& parts) {
  crc_init();
  const unsigned char hdr[10] = {0x1f, 0x8b, 8, 0, 0, 0, 0, 0, 0, 255};  // deflate, no flags, no mtime, OS unknown
  if (fwrite(hdr, 1, 10, f) != 10) return false;
  size_t total = 0;
  for (auto& p : parts) total += p.second;
  uint32_t crc = 0;
  size_t done = 0;
  size_t pi = 0, off = 0;
  std::vector<unsigned char> blk;
  do {
    const size_t len = std::min<size_t>(65535, total - done);
    blk.clear();
    blk.push_back(done + len == total ? 1 : 0);  // BFINAL, BTYPE 00
    put16(blk, (uint32_t)len);
    put16(blk, (uint32_t)(~len & 0xFFFF));
    if (fwrite(blk.data(), 1, blk.size(), f) != blk.size()) return false;
    size_t left = len;
    while (left > 0) {
      const size_t take = std::min(left, parts[pi].second - off);
      const unsigned char* src = (const unsigned char*)parts[pi].first + off;
      if (fwrite(src, 1, take, f) != take) return false;
      crc = crc_update(crc, src, take);
      off += take;
      left -= take;
      if (off == parts[pi].second) {
        pi++;
        off = 0;
      }
    }
    done += len;
  } while (done < total);
  std::vector<unsigned char> tr;
  put32(tr, crc);
  put32(tr, (uint32_t)(total & 0xFFFFFFFFu));
  return fwrite(tr.data(), 1, tr.size(), f) == tr.size();
}

// UniHeader (iogrids.cpp:38-44): 288 bytes with the 8-byte timestamp aligned
struct UniHeader {
  int dimX, dimY, dimZ;
  int gridType, elementType, bytesPerElement;
  char info[252];
  int dimT;
  unsigned long long timestamp;
};
static_assert(sizeof(UniHeader) == 288, "UniHeader layout");

// GridBase::GridType flags (grid.h:29)
int grid_type_flags(int kind) {
  switch (kind) {
    case MG_REAL: return 1;
    case MG_INT: return 2;
    case MG_VEC3: return 4;
    case MG_MAC: return 4 | 8;
    case MG_FLAGS: return 2 | 32;
    case MG_LEVELSET: return 1 | 16;
  }
  return 0;
}

// cnpy's .npy header: magic, version 1.0, the dict padded with spaces to a
// 16-byte boundary and ended by a newline
std::vector<unsigned char> npy_header(const char* descr, const std::vector<size_t>& shape) {
  std::string d = std::string("{'descr': '") + descr + "', 'fortran_order': False, 'shape': (";
  for (size_t i = 0; i < shape.size(); i++) d += std::to_string(shape[i]) + ", ";
  d += "), }";
  const size_t pre = 10;
  size_t total = pre + d.size() + 1;
  const size_t pad = (16 - total % 16) % 16;
  d += std::string(pad, ' ');
  d += '\n';
  std::vector<unsigned char> h = {0x93, 'N', 'U', 'M', 'P', 'Y', 1, 0};
  put16(h, (uint32_t)d.size());
  h.insert(h.end(), d.begin(), d.end());
  return h;
}

// an uncompressed zip (PKWARE APPNOTE, method 0) holding one member
bool write_zip_stored(FILE* f, const std::string& member, const std::vector<unsigned char>& head, const void* data,
                      size_t bytes) {
  crc_init();
  const size_t size = head.size() + bytes;
  if (size >= 0xFFFFFFFFull) return false;  // zip64 is not written
  uint32_t crc = crc_update(0, head.data(), head.size());
  crc = crc_update(crc, (const unsigned char*)data, bytes);
  std::vector<unsigned char> lh;
  put32(lh, 0x04034b50);
  put16(lh, 20);  // version needed
  put16(lh, 0);   // flags
  put16(lh, 0);   // stored
  put16(lh, 0);   // time
  put16(lh, 0);   // date
  put32(lh, crc);
  put32(lh, (uint32_t)size);
  put32(lh, (uint32_t)size);
  put16(lh, (uint32_t)member.size());
  put16(lh, 0);
  lh.insert(lh.end(), member.begin(), member.end());
  if (fwrite(lh.data(), 1, lh.size(), f) != lh.size()) return false;
  if (fwrite(head.data(), 1, head.size(), f) != head.size()) return false;
  if (bytes && fwrite(data, 1, bytes, f) != bytes) return false;
  std::vector<unsigned char> cd;
  put32(cd, 0x02014b50);
  put16(cd, 20);  // version made by
  put16(cd, 20);
  put16(cd, 0);
  put16(cd, 0);
  put16(cd, 0);
  put16(cd, 0);
  put32(cd, crc);
  put32(cd, (uint32_t)size);
  put32(cd, (uint32_t)size);
  put16(cd, (uint32_t)member.size());
  put16(cd, 0);  // extra
  put16(cd, 0);  // comment
  put16(cd, 0);  // disk
  put16(cd, 0);  // internal attributes
  put32(cd, 0);  // external attributes
  put32(cd, 0);  // offset of the local header
  cd.insert(cd.end(), member.begin(), member.end());
  const uint32_t cdOffset = (uint32_t)(lh.size() + size);
  std::vector<unsigned char> end;
  put32(end, 0x06054b50);
  put16(end, 0);
  put16(end, 0);
  put16(end, 1);
  put16(end, 1);
  put32(end, (uint32_t)cd.size());
  put32(end, cdOffset);
  put16(end, 0);
  if (fwrite(cd.data(), 1, cd.size(), f) != cd.size()) return false;
  return fwrite(end.data(), 1, end.size(), f) == end.size();
}

}  // namespace

extern "C" int mg_grid_get_info(mg_grid g, int* nx, int* ny, int* nz, int* kind);

extern "C" int mg_grid_save(mg_grid g, const char* path) {
  int nx = 0, ny = 0, nz = 0, kind = 0;
  const int st = mg_grid_get_info(g, &nx, &ny, &nz, &kind);
  if (st) return st;
  if (!path) return set_error(MG_ERR_ARG, "mg_grid_save: null path");
  const std::string name(path);
  const size_t dot = name.find_last_of('.');
  if (dot == std::string::npos) return set_error(MG_ERR_ARG, "file '" + name + "' does not have an extension");
  const std::string ext = name.substr(dot);
  if (ext != ".uni" && ext != ".raw" && ext != ".npz")
    return set_error(MG_ERR_UNSUPPORTED, "file '" + name + "' filetype not supported");
  const int comps = (kind == MG_VEC3 || kind == MG_MAC) ? 3 : 1;
  const size_t cells = (size_t)nx * ny * nz;
  const size_t bytes = cells * comps * 4;
  // the device mirror, in the reference layout, through pinned memory
  void* host = nullptr;
  if (cudaMallocHost(&host, bytes) != cudaSuccess) {
    cudaGetLastError();
    return set_error(MG_ERR_NOMEM, "mg_grid_save: cannot allocate the host staging buffer");
  }
  int rc = mg_grid_download(g, host, bytes);
  if (rc) {
    cudaFreeHost(host);
    return rc;
  }
  FILE* f = fopen(path, "wb");
  if (!f) {
    cudaFreeHost(host);
    const std::string what = ext == ".uni" ? "writeGridUni" : (ext == ".raw" ? "writeGridRaw" : "writeGridNumpy");
    return set_error(MG_ERR_ARG, what + ": can't open file " + name);
  }
  bool ok;
  if (ext == ".uni") {
    UniHeader h;
    memset(&h, 0, sizeof(h));
    h.dimX = nx;
    h.dimY = ny;
    h.dimZ = nz;
    h.dimT = 0;
    h.gridType = grid_type_flags(kind);
    h.elementType = (kind == MG_INT || kind == MG_FLAGS) ? 0 : (comps == 3 ? 2 : 1);
    h.bytesPerElement = comps * 4;
    snprintf(h.info, sizeof(h.info), "%s", "mantaflow_gb300 sm_103a fp1 (device-resident grid)");
    h.timestamp = (unsigned long long)std::chrono::duration_cast<std::chrono::milliseconds>(
                      std::chrono::system_clock::now().time_since_epoch())
                      .count();
    ok = write_gzip(f, {{"MNT3", 4}, {&h, sizeof(h)}, {host, bytes}});
  } else if (ext == ".raw") {
    ok = write_gzip(f, {{host, bytes}});
  } else {
    const char* descr = (kind == MG_INT || kind == MG_FLAGS) ? "<i4" : "<f4";
    ok = write_zip_stored(f, "arr_0.npy", npy_header(descr, {(size_t)nz, (size_t)ny, (size_t)nx, (size_t)comps}), host,
                          bytes);
  }
  ok = (fclose(f) == 0) && ok;
  cudaFreeHost(host);
  if (!ok) return set_error(MG_ERR_ARG, "mg_grid_save: writing '" + name + "' failed");
  return MG_OK;
}
