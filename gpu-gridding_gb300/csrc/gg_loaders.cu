// Dataset loaders on either side of the gridder: the OSKAR binary container
// that holds the challenge's visibility files (.vis), and the FITS cubes that
// hold its W-kernels.  Host code only; the gridder never calls it.
//
// OSKAR binary reader.  The reference reads its datasets through the OSKAR
// binary library (utils/binary/, oskar_binary_create.c:49-306 for the index,
// oskar_binary_read.c:39-101 for reads, oskar_binary_query.c:60-89 for
// look-ups) and two helpers (utils/read_vis.c:31-73).  The container, as its
// own header documents it (utils/binary/private_binary.h:40-160): a 64-byte
// file header ("OSKARBIN\0", format version), then chunks, each a 20-byte tag
// ('T', 0x40 + format version, 'G', element size, flags, data type, group,
// tag, 4-byte little-endian user index, 8-byte little-endian block size),
// optional group and tag name strings (extended tags), the payload and an
// optional little-endian CRC-32C of tag, names and payload.  This file reads
// that layout with its own index and its own CRC-32C (Castagnoli,
// reflected polynomial 0x82F63B78, initial value and final XOR 0xFFFFFFFF);
// writing is not provided.  Entry points keep the reference's names,
// arguments and int* status codes, so a caller of the reference's reader
// links against this library unchanged.
//
// Both are compiled with the CUDA sources but run on the host only.
//
// FITS kernel reader.  The reference reads each W-kernel cube (the real and
// the imaginary part are separate files) with cfitsio
// (utils/read_kernel.c:36-118): a 3-D primary image [planes][csh][csh], the
// header keys OVERSAMP, GRIDSIZE, CELLSIZE and W_SCALE, and the support of
// each plane from column 1 of the binary-table extension W_KERNELS.  This
// file reads those parts of the FITS standard itself (2880-byte records of
// 80-character header cards, big-endian data, BITPIX 8/16/32/64/-32/-64 with
// BSCALE/BZERO, BINTABLE columns of TFORM B/I/J/K/E/D); cfitsio is not used.
#include <cctype>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "gg_internal.h"
#include "../../include/gpugrid_io.h"

struct oskar_Binary {
  FILE* stream = nullptr;
  int bin_version = 0;
  struct Chunk {
    bool extended = false;
    int data_type = 0, id_group = 0, id_tag = 0, user_index = 0;
    std::string name_group, name_tag;
    long long payload_offset = 0;
    size_t payload_size = 0;
    bool has_crc = false;
    uint32_t crc = 0;         // stored CRC-32C of the chunk
    uint32_t crc_head = 0;    // running CRC-32C of tag and names
  };
  std::vector<Chunk> chunks;
};

namespace {

// ---- CRC-32C ---------------------------------------------------------------
struct Crc32c {
  uint32_t t[256];
  Crc32c() {
    for (uint32_t i = 0; i < 256; ++i) {
      uint32_t c = i;
      for (int k = 0; k < 8; ++k) c = (c >> 1) ^ ((c & 1u) ? 0x82F63B78u : 0u);
      t[i] = c;
    }
  }
  // Running register (not yet complemented): start from 0xFFFFFFFF, feed
  // bytes, complement at the end.
  uint32_t feed(uint32_t reg, const void* data, size_t n) const {
    const unsigned char* p = (const unsigned char*)data;
    for (size_t i = 0; i < n; ++i) reg = (reg >> 8) ^ t[(reg ^ p[i]) & 0xFFu];
    return reg;
  }
};
const Crc32c& crc_table() {
  static const Crc32c c;
  return c;
}

bool host_is_little_endian() {
  const uint16_t x = 1;
  unsigned char b;
  std::memcpy(&b, &x, 1);
  return b == 1;
}

uint64_t le_u64(const unsigned char* p) {
  uint64_t v = 0;
  for (int i = 7; i >= 0; --i) v = (v << 8) | p[i];
  return v;
}
uint32_t le_u32(const unsigned char* p) {
  return (uint32_t)p[0] | ((uint32_t)p[1] << 8) | ((uint32_t)p[2] << 16) |
         ((uint32_t)p[3] << 24);
}

// OSKAR type codes (utils/binary/oskar_binary_data_types.h:46-61).
constexpr int kChar = 0x01, kInt = 0x02, kSingle = 0x04, kDouble = 0x08;
constexpr int kComplex = 0x20, kMatrix = 0x40;
constexpr int kFormatVersion = 2;

// Reads and indexes every chunk; returns 0 or an OSKAR_ERR_BINARY_* code.
int index_file(oskar_Binary* h) {
  unsigned char head[64];
  if (std::fread(head, 1, 64, h->stream) != 64)
    return OSKAR_ERR_BINARY_FILE_INVALID;
  if (std::memcmp(head, "OSKARBIN", 9) != 0)
    return OSKAR_ERR_BINARY_FILE_INVALID;
  h->bin_version = head[9];
  if (h->bin_version < 1 || h->bin_version > kFormatVersion)
    return OSKAR_ERR_BINARY_VERSION_UNKNOWN;
  const Crc32c& crc = crc_table();
  for (;;) {
    unsigned char tag[20];
    const size_t got = std::fread(tag, 1, 20, h->stream);
    if (got == 0) break;                       // clean end of file
    if (got != 20) return OSKAR_ERR_BINARY_FILE_INVALID;
    const unsigned flags = tag[4];
    if (tag[0] != 'T' || tag[2] != 'G' || (flags & 0x1Fu) != 0)
      return OSKAR_ERR_BINARY_FILE_INVALID;
    const int version = (int)tag[1] - 0x40;
    if (version < 1 || version > kFormatVersion)
      return OSKAR_ERR_BINARY_VERSION_UNKNOWN;
    const int dtype = tag[5];
    if (version > 1) {
      // Payload byte order: this reader takes little-endian payloads only
      // (every host it targets is little-endian).
      if ((flags & 0x20u) || !host_is_little_endian())
        return OSKAR_ERR_BINARY_ENDIAN_MISMATCH;
      int elem = tag[3];
      if (dtype & kMatrix) elem /= 4;
      if (dtype & kComplex) elem /= 2;
      if (dtype & kChar) {
        if (elem != 1) return OSKAR_ERR_BINARY_FORMAT_BAD;
      } else if (dtype & kInt) {
        if (elem != (int)sizeof(int)) return OSKAR_ERR_BINARY_INT_UNKNOWN;
      } else if (dtype & kSingle) {
        if (elem != 4) return OSKAR_ERR_BINARY_FLOAT_UNKNOWN;
      } else if (dtype & kDouble) {
        if (elem != 8) return OSKAR_ERR_BINARY_DOUBLE_UNKNOWN;
      } else {
        return OSKAR_ERR_BINARY_TYPE_UNKNOWN;
      }
    }
    oskar_Binary::Chunk c;
    c.data_type = dtype;
    c.id_group = tag[6];
    c.id_tag = tag[7];
    c.user_index = (int)le_u32(tag + 8);
    const uint64_t block = le_u64(tag + 12);
    c.has_crc = (flags & 0x40u) != 0;
    c.extended = (flags & 0x80u) != 0;
    uint32_t reg = crc.feed(0xFFFFFFFFu, tag, 20);
    uint64_t names = 0;
    if (c.extended) {
      const size_t lg = tag[6], lt = tag[7];
      std::vector<char> g(lg + 1, 0), t(lt + 1, 0);
      if ((lg && std::fread(g.data(), 1, lg, h->stream) != lg) ||
          (lt && std::fread(t.data(), 1, lt, h->stream) != lt))
        return OSKAR_ERR_BINARY_FILE_INVALID;
      reg = crc.feed(reg, g.data(), lg);
      reg = crc.feed(reg, t.data(), lt);
      c.name_group.assign(g.data());
      c.name_tag.assign(t.data());
      names = lg + lt;
    }
    const uint64_t extra = names + (c.has_crc ? 4u : 0u);
    if (block < extra) return OSKAR_ERR_BINARY_FILE_INVALID;
    c.payload_size = (size_t)(block - extra);
    c.payload_offset = (long long)ftello(h->stream);
    c.crc_head = reg;
    if (fseeko(h->stream, (off_t)c.payload_size, SEEK_CUR) != 0)
      return OSKAR_ERR_BINARY_FILE_INVALID;
    if (c.has_crc) {
      unsigned char b[4];
      if (std::fread(b, 1, 4, h->stream) != 4)
        return OSKAR_ERR_BINARY_FILE_INVALID;
      c.crc = le_u32(b);
    }
    h->chunks.push_back(std::move(c));
  }
  // As in the reference, a last payload cut short by the end of the file
  // is indexed and fails when it is read (OSKAR_ERR_BINARY_READ_FAIL).
  return 0;
}

}  // namespace

extern "C" {

GG_API oskar_Binary* oskar_binary_create(const char* filename, char mode,
                                         int* status) {
  if (!status) return nullptr;
  if (*status) return nullptr;
  if (mode != 'r' || !filename) {
    // Writing and appending are not provided by this reader.
    *status = OSKAR_ERR_BINARY_OPEN_FAIL;
    return nullptr;
  }
  FILE* f = std::fopen(filename, "rb");
  if (!f) {
    *status = OSKAR_ERR_BINARY_OPEN_FAIL;
    return nullptr;
  }
  oskar_Binary* h = new oskar_Binary;
  h->stream = f;
  const int r = index_file(h);
  if (r) {
    *status = r;
    std::fclose(f);
    delete h;
    return nullptr;
  }
  return h;
}

GG_API void oskar_binary_free(oskar_Binary* handle) {
  if (!handle) return;
  if (handle->stream) std::fclose(handle->stream);
  delete handle;
}

GG_API int oskar_binary_num_tags(const oskar_Binary* handle) {
  return handle ? (int)handle->chunks.size() : 0;
}

GG_API int oskar_binary_query(const oskar_Binary* handle,
                              unsigned char data_type, unsigned char id_group,
                              unsigned char id_tag, int user_index,
                              size_t* payload_size, int* status) {
  if (!status || *status) return 0;
  if (!handle) {
    *status = OSKAR_ERR_BINARY_NOT_OPEN_FOR_READ;
    return -1;
  }
  for (size_t i = 0; i < handle->chunks.size(); ++i) {
    const oskar_Binary::Chunk& c = handle->chunks[i];
    if (!c.extended && (c.data_type == (int)data_type || !data_type) &&
        c.id_group == (int)id_group && c.id_tag == (int)id_tag &&
        c.user_index == user_index) {
      if (payload_size) *payload_size = c.payload_size;
      return (int)i;
    }
  }
  *status = OSKAR_ERR_BINARY_TAG_NOT_FOUND;
  return -1;
}

GG_API void oskar_binary_read_block(oskar_Binary* handle, int chunk_index,
                                    size_t data_size, void* data,
                                    int* status) {
  if (!status || *status) return;
  if (!handle) {
    *status = OSKAR_ERR_BINARY_NOT_OPEN_FOR_READ;
    return;
  }
  if (chunk_index < 0 || chunk_index >= (int)handle->chunks.size()) {
    *status = OSKAR_ERR_BINARY_TAG_OUT_OF_RANGE;
    return;
  }
  const oskar_Binary::Chunk& c = handle->chunks[chunk_index];
  if (c.payload_size == 0) return;
  if (!data || data_size < c.payload_size) {
    *status = OSKAR_ERR_BINARY_MEMORY_NOT_ALLOCATED;
    return;
  }
  if (fseeko(handle->stream, (off_t)c.payload_offset, SEEK_SET) != 0) {
    *status = OSKAR_ERR_BINARY_SEEK_FAIL;
    return;
  }
  // In pieces of at most 512 MiB (some C libraries limit one fread).
  const size_t piece = size_t(1) << 29;
  unsigned char* p = (unsigned char*)data;
  for (size_t left = c.payload_size; left > 0;) {
    const size_t n = left < piece ? left : piece;
    if (std::fread(p, 1, n, handle->stream) != n) {
      *status = OSKAR_ERR_BINARY_READ_FAIL;
      return;
    }
    p += n;
    left -= n;
  }
  if (c.has_crc) {
    const uint32_t reg =
        crc_table().feed(c.crc_head, data, c.payload_size) ^ 0xFFFFFFFFu;
    if (reg != c.crc) *status = OSKAR_ERR_BINARY_CRC_FAIL;
  }
}

GG_API void oskar_binary_read(oskar_Binary* handle, unsigned char data_type,
                              unsigned char id_group, unsigned char id_tag,
                              int user_index, size_t data_size, void* data,
                              int* status) {
  if (!status || *status) return;
  const int i = oskar_binary_query(handle, data_type, id_group, id_tag,
                                   user_index, nullptr, status);
  oskar_binary_read_block(handle, i, data_size, data, status);
}

GG_API void oskar_binary_read_int(oskar_Binary* handle, unsigned char id_group,
                                  unsigned char id_tag, int user_index,
                                  int* value, int* status) {
  oskar_binary_read(handle, kInt, id_group, id_tag, user_index, sizeof(int),
                    value, status);
}

GG_API void oskar_binary_read_double(oskar_Binary* handle,
                                     unsigned char id_group,
                                     unsigned char id_tag, int user_index,
                                     double* value, int* status) {
  oskar_binary_read(handle, kDouble, id_group, id_tag, user_index,
                    sizeof(double), value, status);
}

// utils/read_vis.c:31-47: the baseline coordinates of one visibility block
// (group 12, tags 4, 5, 6, user index = block).
GG_API void gg_vis_read_coords(oskar_Binary* h, int i_block, int precision,
                               size_t num_coords, void* uu, void* vv,
                               void* ww, int* status) {
  if (!status || *status) return;
  if (precision != OSKAR_DOUBLE && precision != OSKAR_SINGLE) {
    *status = OSKAR_ERR_BINARY_TYPE_UNKNOWN;
    return;
  }
  const size_t bytes =
      (precision == OSKAR_DOUBLE ? sizeof(double) : sizeof(float)) *
      num_coords;
  oskar_binary_read(h, (unsigned char)precision, OSKAR_TAG_GROUP_VIS_BLOCK,
                    OSKAR_VIS_BLOCK_TAG_BASELINE_UU, i_block, bytes, uu,
                    status);
  oskar_binary_read(h, (unsigned char)precision, OSKAR_TAG_GROUP_VIS_BLOCK,
                    OSKAR_VIS_BLOCK_TAG_BASELINE_VV, i_block, bytes, vv,
                    status);
  oskar_binary_read(h, (unsigned char)precision, OSKAR_TAG_GROUP_VIS_BLOCK,
                    OSKAR_VIS_BLOCK_TAG_BASELINE_WW, i_block, bytes, ww,
                    status);
}

// utils/read_vis.c:49-73: metres to wavelengths, scale = freq / c formed in
// FP64, applied in the arrays' precision (FP32 arrays take the FP32-rounded
// scale).
GG_API void gg_vis_scale_coords(double freq_hz, int precision,
                                size_t num_coords, void* uu, void* vv,
                                void* ww) {
  const double scale = freq_hz / 299792458.0;
  if (precision == OSKAR_DOUBLE) {
    double *u = (double*)uu, *v = (double*)vv, *w = (double*)ww;
    for (size_t i = 0; i < num_coords; ++i) {
      u[i] *= scale; v[i] *= scale; w[i] *= scale;
    }
  } else if (precision == OSKAR_SINGLE) {
    const float s = (float)scale;
    float *u = (float*)uu, *v = (float*)vv, *w = (float*)ww;
    for (size_t i = 0; i < num_coords; ++i) {
      u[i] *= s; v[i] *= s; w[i] *= s;
    }
  }
}

}  // extern "C"

// ===========================================================================
// FITS kernel cubes
// ===========================================================================
namespace {

constexpr size_t kFitsBlock = 2880;

struct FitsHdu {
  std::vector<std::pair<std::string, std::string>> cards;  // key, raw value
  long long data_offset = 0;   // first data byte
  long long data_bytes = 0;    // without padding
  bool find(const char* key, std::string* value) const {
    for (const auto& kv : cards)
      if (kv.first == key) {
        *value = kv.second;
        return true;
      }
    return false;
  }
};

std::string trim(const std::string& s) {
  size_t a = 0, b = s.size();
  while (a < b && std::isspace((unsigned char)s[a])) ++a;
  while (b > a && std::isspace((unsigned char)s[b - 1])) --b;
  return s.substr(a, b - a);
}

// The value field of a card (columns 11-80 after "= "), without its
// comment; string values lose their quotes and trailing blanks.
std::string card_value(const char* card) {
  std::string v(card + 10, 70);
  std::string out;
  size_t i = 0;
  while (i < v.size() && v[i] == ' ') ++i;
  if (i < v.size() && v[i] == '\'') {
    for (++i; i < v.size(); ++i) {
      if (v[i] == '\'') {
        if (i + 1 < v.size() && v[i + 1] == '\'') {
          out += '\'';
          ++i;
          continue;
        }
        break;
      }
      out += v[i];
    }
    return trim(out);
  }
  const size_t slash = v.find('/', i);
  return trim(v.substr(i, slash == std::string::npos ? std::string::npos
                                                      : slash - i));
}

bool to_long(const std::string& s, long long* out) {
  if (s.empty()) return false;
  char* end = nullptr;
  const long long v = std::strtoll(s.c_str(), &end, 10);
  if (*end) return false;
  *out = v;
  return true;
}

bool to_double(std::string s, double* out) {
  if (s.empty()) return false;
  for (char& c : s)
    if (c == 'D' || c == 'd') c = 'E';   // FORTRAN exponent
  char* end = nullptr;
  const double v = std::strtod(s.c_str(), &end);
  if (*end) return false;
  *out = v;
  return true;
}

// Reads one HDU's header at the current position; returns false at end of
// file or on a malformed header.
bool read_hdu(FILE* f, FitsHdu* h) {
  char block[kFitsBlock];
  bool ended = false;
  while (!ended) {
    if (std::fread(block, 1, kFitsBlock, f) != kFitsBlock) return false;
    for (size_t c = 0; c < kFitsBlock; c += 80) {
      const char* card = block + c;
      const std::string key = trim(std::string(card, 8));
      if (key == "END") {
        ended = true;
        break;
      }
      if (card[8] == '=' && card[9] == ' ')
        h->cards.emplace_back(key, card_value(card));
    }
  }
  h->data_offset = (long long)ftello(f);
  std::string v;
  long long bitpix = 0, naxis = 0, pcount = 0, gcount = 1, n = 1;
  if (!h->find("BITPIX", &v) || !to_long(v, &bitpix)) return false;
  if (!h->find("NAXIS", &v) || !to_long(v, &naxis)) return false;
  if (naxis < 0 || naxis > 999) return false;
  for (long long i = 1; i <= naxis; ++i) {
    long long d = 0;
    if (!h->find(("NAXIS" + std::to_string(i)).c_str(), &v) ||
        !to_long(v, &d) || d < 0)
      return false;
    n *= d;
  }
  if (naxis == 0) n = 0;
  if (h->find("PCOUNT", &v)) to_long(v, &pcount);
  if (h->find("GCOUNT", &v)) to_long(v, &gcount);
  h->data_bytes = (long long)(std::llabs(bitpix) / 8) * gcount * (pcount + n);
  return true;
}

bool skip_data(FILE* f, const FitsHdu& h) {
  const long long padded =
      (h.data_bytes + (long long)kFitsBlock - 1) / (long long)kFitsBlock *
      (long long)kFitsBlock;
  return fseeko(f, (off_t)(h.data_offset + padded), SEEK_SET) == 0;
}

// Big-endian element at p of a FITS type of `bytes` bytes: integer
// (signed; 8-bit unsigned) or IEEE floating point, as a double.
double be_value(const unsigned char* p, int bytes, bool is_float) {
  uint64_t u = 0;
  for (int i = 0; i < bytes; ++i) u = (u << 8) | p[i];
  if (is_float) {
    if (bytes == 4) {
      const uint32_t w = (uint32_t)u;
      float x;
      std::memcpy(&x, &w, 4);
      return x;
    }
    double x;
    std::memcpy(&x, &u, 8);
    return x;
  }
  switch (bytes) {
    case 1: return (double)(uint8_t)u;
    case 2: return (double)(int16_t)(uint16_t)u;
    case 4: return (double)(int32_t)(uint32_t)u;
    default: return (double)(int64_t)u;
  }
}

bool name_is(const FitsHdu& h, const char* key, const char* want) {
  std::string v;
  if (!h.find(key, &v)) return false;
  if (v.size() != std::strlen(want)) return false;
  for (size_t i = 0; i < v.size(); ++i)
    if (std::toupper((unsigned char)v[i]) != want[i]) return false;
  return true;
}

int fits_fail(int* status, const char* msg) {
  *status = 1;
  gg::record_error(GG_ERR_INVALID_ARG, msg);
  return 1;
}

}  // namespace

extern "C" GG_API void* gg_read_kernel(const char* file_name, int precision,
                                       int* conv_size_half, int* num_w_planes,
                                       int** support, int* oversample,
                                       int* grid_size, double* cellsize_rad,
                                       double* w_scale, int* status) {
  if (!status || *status) return nullptr;
  if (precision != OSKAR_SINGLE && precision != OSKAR_DOUBLE) {
    fits_fail(status, "precision must be OSKAR_SINGLE or OSKAR_DOUBLE");
    return nullptr;
  }
  FILE* f = file_name ? std::fopen(file_name, "rb") : nullptr;
  if (!f) {
    fits_fail(status, "cannot open the kernel FITS file");
    return nullptr;
  }
  void* data = nullptr;
  FitsHdu prim;
  std::string v;
  long long bitpix = 0, naxis = 0, d[3] = {0, 0, 0};
  double bscale = 1.0, bzero = 0.0;
  long long key_os = 0, key_gs = 0;
  double key_cell = 0.0, key_ws = 0.0;
  size_t n = 0;
  int bytes = 0;
  std::vector<unsigned char> raw;
  if (!read_hdu(f, &prim) || !prim.find("SIMPLE", &v) || v != "T") {
    fits_fail(status, "not a FITS file");
    goto done;
  }
  prim.find("BITPIX", &v);
  to_long(v, &bitpix);
  prim.find("NAXIS", &v);
  to_long(v, &naxis);
  if (naxis != 3) {
    fits_fail(status, "Need a 3D kernel FITS cube.");
    goto done;
  }
  for (int i = 0; i < 3; ++i) {
    prim.find(("NAXIS" + std::to_string(i + 1)).c_str(), &v);
    to_long(v, &d[i]);
  }
  if (!prim.find("OVERSAMP", &v) || !to_long(v, &key_os)) {
    fits_fail(status, "Missing 'OVERSAMP' FITS header keyword.");
    goto done;
  }
  if (!prim.find("GRIDSIZE", &v) || !to_long(v, &key_gs)) {
    fits_fail(status, "Missing 'GRIDSIZE' FITS header keyword.");
    goto done;
  }
  if (!prim.find("CELLSIZE", &v) || !to_double(v, &key_cell)) {
    fits_fail(status, "Missing 'CELLSIZE' FITS header keyword.");
    goto done;
  }
  if (!prim.find("W_SCALE", &v) || !to_double(v, &key_ws)) {
    fits_fail(status, "Missing 'W_SCALE' FITS header keyword.");
    goto done;
  }
  if (prim.find("BSCALE", &v)) to_double(v, &bscale);
  if (prim.find("BZERO", &v)) to_double(v, &bzero);
  if (bitpix != 8 && bitpix != 16 && bitpix != 32 && bitpix != 64 &&
      bitpix != -32 && bitpix != -64) {
    fits_fail(status, "unsupported BITPIX");
    goto done;
  }
  *conv_size_half = (int)d[0];
  *num_w_planes = (int)d[2];
  *oversample = (int)key_os;
  *grid_size = (int)key_gs;
  *cellsize_rad = key_cell;
  *w_scale = key_ws;
  // Pixels in file order (NAXIS1 fastest), converted to the precision.
  n = (size_t)(d[0] * d[1] * d[2]);
  bytes = (int)(std::llabs(bitpix) / 8);
  raw.resize(n * (size_t)bytes);
  if (fseeko(f, (off_t)prim.data_offset, SEEK_SET) != 0 ||
      (n && std::fread(raw.data(), 1, raw.size(), f) != raw.size())) {
    fits_fail(status, "kernel cube data cut short");
    goto done;
  }
  data = std::calloc(n ? n : 1, precision == OSKAR_DOUBLE ? 8 : 4);
  if (!data) {
    fits_fail(status, "out of host memory");
    goto done;
  }
  for (size_t i = 0; i < n; ++i) {
    double x = be_value(&raw[i * bytes], bytes, bitpix < 0);
    if (bscale != 1.0 || bzero != 0.0) x = bzero + bscale * x;
    if (precision == OSKAR_DOUBLE) ((double*)data)[i] = x;
    else ((float*)data)[i] = (float)x;
  }
  // Supports: column 1 of the W_KERNELS binary table, the first
  // num_w_planes elements in (row, element) order.
  if (support) {
    *support = (int*)std::calloc((size_t)(d[2] > 0 ? d[2] : 1), sizeof(int));
    if (!skip_data(f, prim)) {
      fits_fail(status, "Missing 'W_KERNELS' FITS binary table.");
      goto done;
    }
    for (;;) {
      FitsHdu ext;
      if (!read_hdu(f, &ext)) {
        fits_fail(status, "Missing 'W_KERNELS' FITS binary table.");
        goto done;
      }
      if (name_is(ext, "XTENSION", "BINTABLE") &&
          (name_is(ext, "EXTNAME", "W_KERNELS") ||
           name_is(ext, "HDUNAME", "W_KERNELS"))) {
        long long row_bytes = 0, rows = 0, fields = 0;
        ext.find("NAXIS1", &v); to_long(v, &row_bytes);
        ext.find("NAXIS2", &v); to_long(v, &rows);
        ext.find("TFIELDS", &v); to_long(v, &fields);
        std::string form;
        if (fields < 1 || !ext.find("TFORM1", &form)) {
          fits_fail(status, "Unable to read kernel support sizes.");
          goto done;
        }
        // TFORM1 = [repeat]type.
        size_t k = 0;
        long long repeat = 0;
        while (k < form.size() && std::isdigit((unsigned char)form[k]))
          repeat = repeat * 10 + (form[k++] - '0');
        if (k == 0) repeat = 1;
        const char type = k < form.size() ? form[k] : ' ';
        int eb = 0;
        bool fl = false;
        switch (type) {
          case 'B': eb = 1; break;
          case 'I': eb = 2; break;
          case 'J': eb = 4; break;
          case 'K': eb = 8; break;
          case 'E': eb = 4; fl = true; break;
          case 'D': eb = 8; fl = true; break;
          default: break;
        }
        double tscal = 1.0, tzero = 0.0;
        if (ext.find("TSCAL1", &v)) to_double(v, &tscal);
        if (ext.find("TZERO1", &v)) to_double(v, &tzero);
        if (!eb || repeat < 1 || repeat * rows < d[2] ||
            (long long)eb * repeat > row_bytes) {
          fits_fail(status, "Unable to read kernel support sizes.");
          goto done;
        }
        std::vector<unsigned char> row((size_t)row_bytes);
        long long got = 0;
        for (long long r = 0; r < rows && got < d[2]; ++r) {
          if (fseeko(f, (off_t)(ext.data_offset + r * row_bytes),
                     SEEK_SET) != 0 ||
              std::fread(row.data(), 1, row.size(), f) != row.size()) {
            fits_fail(status, "Unable to read kernel support sizes.");
            goto done;
          }
          for (long long e = 0; e < repeat && got < d[2]; ++e) {
            double x = be_value(&row[(size_t)(e * eb)], eb, fl);
            x = tzero + tscal * x;
            (*support)[got++] = (int)std::lround(x);
          }
        }
        break;
      }
      if (!skip_data(f, ext)) {
        fits_fail(status, "Missing 'W_KERNELS' FITS binary table.");
        goto done;
      }
    }
  }
done:
  std::fclose(f);
  if (*status) {
    // On failure nothing is handed to the caller.
    std::free(data);
    data = nullptr;
    if (support && *support) {
      std::free(*support);
      *support = nullptr;
    }
  }
  return data;
}
