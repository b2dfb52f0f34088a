// vcpmat.cu -- portable matrix files (the .vcpmat format of
// vcp/vcp_portable_fio.hpp: save_portable / load_portable), for moving
// operands and results between the reference's CPU programs and GPU runs.
//
// Layout (all integers little-endian; vcp_portable_fio.hpp:51-58, 385-443):
//   "VCPMAT2\0" | version u32 = 2 | type u32 | layout u32 = 1 (column-major)
//   | reserved u32 = 0 | rows u64 | columns u64 | payload bytes u64
//   | payload (column-major elements) | CRC-64 u64
// Element types (:60-66): 1 int32, 2 double, 3 interval<double> {lower,
// upper}, 4 kv::dd {a1, a2}, 5 interval<kv::dd> {lo.a1, lo.a2, up.a1, up.a2};
// doubles as their binary64 bit patterns.  The CRC (:92-108) covers header
// and payload: polynomial 0x42f0e1eba9ea3693 (ECMA-182), most significant
// bit first, initial value 0, no final xor -- computed here with a 256-entry
// table, one byte per step (the same remainder as the reference's bit loop).
// Files are written to "<name>.vcpmat.tmp" and renamed (:476-516); a load
// checks magic, version, layout, reserved field, type, sizes, payload size,
// CRC and trailing bytes as the reference does (:409-565).
//
// The payload of each type is the in-memory layout of its kv type on a
// little-endian machine, so the device forms stream a file to or from HBM in
// chunks through pinned staging buffers (the CRC runs over the same bytes on
// the host while the previous chunk copies).
#include <climits>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "common.cuh"

namespace vcpcu {
namespace {

const unsigned char kMagic[8] = {'V', 'C', 'P', 'M', 'A', 'T', '2', '\0'};
constexpr uint32_t kVersion = 2, kColumnMajor = 1;
constexpr uint64_t kPoly = 0x42f0e1eba9ea3693ULL;

struct CrcTable {
  uint64_t t[256];
  CrcTable() {
    for (int b = 0; b < 256; ++b) {
      uint64_t c = (uint64_t)b << 56;
      for (int k = 0; k < 8; ++k) c = (c & 0x8000000000000000ULL) ? (c << 1) ^ kPoly : c << 1;
      t[b] = c;
    }
  }
};
const CrcTable& crc_table() {
  static const CrcTable tab;
  return tab;
}
void crc_update(uint64_t& crc, const unsigned char* p, size_t n) {
  const uint64_t* t = crc_table().t;
  uint64_t c = crc;
  for (size_t i = 0; i < n; ++i) c = (c << 8) ^ t[(c >> 56) ^ p[i]];
  crc = c;
}

size_t elem_bytes(int type) {
  switch (type) {
    case VCPCU_MAT_INT32: return 4;
    case VCPCU_MAT_DOUBLE: return 8;
    case VCPCU_MAT_INTERVAL: return 16;
    case VCPCU_MAT_DD: return 16;
    case VCPCU_MAT_INTERVAL_DD: return 32;
    default: return 0;
  }
}

void put32(unsigned char* p, uint32_t v) {
  for (int i = 0; i < 4; ++i) p[i] = (unsigned char)(v >> (8 * i));
}
void put64(unsigned char* p, uint64_t v) {
  for (int i = 0; i < 8; ++i) p[i] = (unsigned char)(v >> (8 * i));
}
uint32_t get32(const unsigned char* p) {
  uint32_t v = 0;
  for (int i = 0; i < 4; ++i) v |= (uint32_t)p[i] << (8 * i);
  return v;
}
uint64_t get64(const unsigned char* p) {
  uint64_t v = 0;
  for (int i = 0; i < 8; ++i) v |= (uint64_t)p[i] << (8 * i);
  return v;
}

bool little_endian() {
  const uint32_t one = 1;
  unsigned char b;
  std::memcpy(&b, &one, 1);
  return b == 1;
}

int io_fail(const char* fmt, const std::string& file) {
  set_error(fmt, file.c_str());
  return VCPCU_ERR_IO;
}

struct File {
  FILE* f = nullptr;
  ~File() {
    if (f) std::fclose(f);
  }
};

// Header of `file`: checks everything the reference's read_header and
// check_payload_size check; *type, *rows, *cols receive the values.
int read_header(FILE* f, const std::string& file, uint64_t& crc, int* type, int* rows, int* cols) {
  unsigned char h[48];
  if (std::fread(h, 1, 48, f) != 48) return io_fail("vcpmat: cannot read the header of %s", file);
  crc_update(crc, h, 48);
  if (std::memcmp(h, kMagic, 8) != 0) return io_fail("vcpmat: invalid magic in %s", file);
  if (get32(h + 8) != kVersion) return io_fail("vcpmat: unsupported version in %s", file);
  const uint32_t t = get32(h + 12);
  if (get32(h + 16) != kColumnMajor) return io_fail("vcpmat: unsupported layout in %s", file);
  if (get32(h + 20) != 0) return io_fail("vcpmat: invalid reserved field in %s", file);
  const uint64_t r = get64(h + 24), c = get64(h + 32), pb = get64(h + 40);
  if ((r == 0) != (c == 0)) return io_fail("vcpmat: invalid zero matrix size in %s", file);
  if (r > (uint64_t)INT_MAX || c > (uint64_t)INT_MAX || (r && c > (uint64_t)INT_MAX / r))
    return io_fail("vcpmat: matrix is too large in %s", file);
  const size_t eb = elem_bytes((int)t);
  if (t > 5 || eb == 0) return io_fail("vcpmat: unsupported type id in %s", file);
  if (pb != r * c * eb) return io_fail("vcpmat: payload byte size mismatch in %s", file);
  *type = (int)t;
  *rows = (int)r;
  *cols = (int)c;
  return VCPCU_OK;
}

// Trailer: the stored CRC must match and nothing may follow it.
int read_trailer(FILE* f, const std::string& file, uint64_t crc) {
  unsigned char b[8];
  if (std::fread(b, 1, 8, f) != 8) return io_fail("vcpmat: cannot read the CRC64 of %s", file);
  if (get64(b) != crc) return io_fail("vcpmat: CRC64 mismatch in %s", file);
  if (std::fgetc(f) != EOF) return io_fail("vcpmat: trailing data after CRC64 in %s", file);
  return VCPCU_OK;
}

int check_args(const char* name, int type, int rows, int cols) {
  if (!name) {
    set_error("vcpmat: null file name");
    return VCPCU_ERR_INVALID_ARG;
  }
  if (elem_bytes(type) == 0) {
    set_error("vcpmat: unknown element type %d", type);
    return VCPCU_ERR_INVALID_ARG;
  }
  if (rows < 0 || cols < 0 || ((rows == 0) != (cols == 0))) {
    set_error("vcpmat: invalid matrix size %d x %d", rows, cols);
    return VCPCU_ERR_INVALID_ARG;
  }
  if (type != VCPCU_MAT_INT32 && !little_endian()) {
    set_error("vcpmat: this build writes payloads from little-endian memory only");
    return VCPCU_ERR_UNSUPPORTED;
  }
  return VCPCU_OK;
}

// Writes header, payload (by the callback, which hands out consecutive
// chunks) and CRC into <name>.vcpmat.tmp, then renames it.
template <class Chunks>
int save_file(const char* name, int type, int rows, int cols, Chunks next_chunk) {
  const std::string file = std::string(name) + ".vcpmat", tmp = file + ".tmp";
  const uint64_t payload = (uint64_t)rows * cols * elem_bytes(type);
  int st = VCPCU_OK;
  {
    File out;
    out.f = std::fopen(tmp.c_str(), "wb");
    if (!out.f) return io_fail("vcpmat: cannot open output file %s", tmp);
    unsigned char h[48];
    std::memcpy(h, kMagic, 8);
    put32(h + 8, kVersion);
    put32(h + 12, (uint32_t)type);
    put32(h + 16, kColumnMajor);
    put32(h + 20, 0);
    put64(h + 24, (uint64_t)rows);
    put64(h + 32, (uint64_t)cols);
    put64(h + 40, payload);
    uint64_t crc = 0;
    crc_update(crc, h, 48);
    if (std::fwrite(h, 1, 48, out.f) != 48) st = io_fail("vcpmat: failed to write %s", tmp);
    uint64_t done = 0;
    while (st == VCPCU_OK && done < payload) {
      const unsigned char* p = nullptr;
      size_t n = 0;
      if ((st = next_chunk(done, &p, &n))) break;
      crc_update(crc, p, n);
      if (std::fwrite(p, 1, n, out.f) != n) st = io_fail("vcpmat: failed to write %s", tmp);
      done += n;
    }
    if (st == VCPCU_OK) {
      unsigned char b[8];
      put64(b, crc);
      if (std::fwrite(b, 1, 8, out.f) != 8) st = io_fail("vcpmat: failed to write %s", tmp);
    }
    if (std::fclose(out.f) != 0 && st == VCPCU_OK)
      st = io_fail("vcpmat: failed to close output file %s", tmp);
    out.f = nullptr;
  }
  if (st == VCPCU_OK && std::rename(tmp.c_str(), file.c_str()) != 0)
    st = io_fail("vcpmat: failed to replace output file %s", file);
  if (st != VCPCU_OK) std::remove(tmp.c_str());
  return st;
}

// Opens <name>.vcpmat and checks its header against the expected type and
// size.
int open_for_load(const char* name, int type, int rows, int cols, File& in, std::string& file,
                  uint64_t& crc) {
  file = std::string(name) + ".vcpmat";
  in.f = std::fopen(file.c_str(), "rb");
  if (!in.f) return io_fail("vcpmat: cannot open input file %s", file);
  int ft, fr, fc;
  int st = read_header(in.f, file, crc, &ft, &fr, &fc);
  if (st) return st;
  if (ft != type) {
    set_error("vcpmat: data type mismatch in %s: file type %d, requested %d", file.c_str(), ft,
              type);
    return VCPCU_ERR_IO;
  }
  if (fr != rows || fc != cols) {
    set_error("vcpmat: %s holds a %d x %d matrix, the caller expects %d x %d", file.c_str(), fr,
              fc, rows, cols);
    return VCPCU_ERR_INVALID_ARG;
  }
  return VCPCU_OK;
}

constexpr size_t kChunk = 64u << 20;  // staging chunk of the device forms

struct Pinned {
  void* p = nullptr;
  ~Pinned() {
    if (p) cudaFreeHost(p);
  }
};

}  // namespace
}  // namespace vcpcu

using namespace vcpcu;

extern "C" int vcpcu_vcpmat_save(const char* name, int type, int rows, int cols,
                                 const void* data) {
  clear_error();
  int st = check_args(name, type, rows, cols);
  if (st) return st;
  if (rows > 0 && !data) {
    set_error("vcpmat: null data");
    return VCPCU_ERR_INVALID_ARG;
  }
  const unsigned char* base = (const unsigned char*)data;
  const uint64_t total = (uint64_t)rows * cols * elem_bytes(type);
  return save_file(name, type, rows, cols,
                   [&](uint64_t done, const unsigned char** p, size_t* n) {
                     *p = base + done;
                     *n = (size_t)(total - done < kChunk ? total - done : kChunk);
                     return VCPCU_OK;
                   });
}

extern "C" int vcpcu_vcpmat_info(const char* name, int* type, int* rows, int* cols) {
  clear_error();
  if (!name || !type || !rows || !cols) {
    set_error("vcpmat: null argument");
    return VCPCU_ERR_INVALID_ARG;
  }
  const std::string file = std::string(name) + ".vcpmat";
  File in;
  in.f = std::fopen(file.c_str(), "rb");
  if (!in.f) return io_fail("vcpmat: cannot open input file %s", file);
  uint64_t crc = 0;
  return read_header(in.f, file, crc, type, rows, cols);
}

extern "C" int vcpcu_vcpmat_load(const char* name, int type, int rows, int cols, void* data) {
  clear_error();
  int st = check_args(name, type, rows, cols);
  if (st) return st;
  if (rows > 0 && !data) {
    set_error("vcpmat: null data");
    return VCPCU_ERR_INVALID_ARG;
  }
  File in;
  std::string file;
  uint64_t crc = 0;
  if ((st = open_for_load(name, type, rows, cols, in, file, crc))) return st;
  unsigned char* out = (unsigned char*)data;
  const uint64_t total = (uint64_t)rows * cols * elem_bytes(type);
  for (uint64_t done = 0; done < total;) {
    const size_t n = (size_t)(total - done < kChunk ? total - done : kChunk);
    if (std::fread(out + done, 1, n, in.f) != n)
      return io_fail("vcpmat: truncated payload in %s", file);
    crc_update(crc, out + done, n);
    done += n;
  }
  return read_trailer(in.f, file, crc);
}

// Device forms: the matrix lives in device memory with leading dimension ld
// (elements); chunks of whole columns pass through two pinned buffers, the
// copy of one overlapping the file I/O and CRC of the other.
namespace {
struct Staging {
  Pinned buf[2];
  cudaEvent_t ev[2] = {nullptr, nullptr};
  size_t cols_per = 1;
  ~Staging() {
    for (int i = 0; i < 2; ++i)
      if (ev[i]) cudaEventDestroy(ev[i]);
  }
  int init(size_t col) {
    cols_per = kChunk / col > 0 ? kChunk / col : 1;
    for (int b = 0; b < 2; ++b) {
      if (cudaMallocHost(&buf[b].p, cols_per * col) != cudaSuccess) {
        set_error("vcpmat: pinned staging allocation of %zu bytes failed", cols_per * col);
        return VCPCU_ERR_ALLOC;
      }
      VCPCU_CUDA_TRY(cudaEventCreateWithFlags(&ev[b], cudaEventDisableTiming));
    }
    return VCPCU_OK;
  }
};
}  // namespace

extern "C" int vcpcu_vcpmat_save_dev(const char* name, int type, int rows, int cols,
                                     const void* ddata, int ld, void* stream) {
  clear_error();
  int st = check_args(name, type, rows, cols);
  if (st) return st;
  if (rows > 0 && (!ddata || ld < rows)) {
    set_error("vcpmat: null data or ld < rows");
    return VCPCU_ERR_INVALID_ARG;
  }
  if ((st = check_device())) return st;
  cudaStream_t s = (cudaStream_t)stream;
  const size_t eb = elem_bytes(type), col = (size_t)rows * eb;
  Staging stg;
  if (col && (st = stg.init(col))) return st;
  const size_t cp = stg.cols_per;
  const int nchunks = col ? (int)((cols + cp - 1) / cp) : 0;
  const unsigned char* dev = (const unsigned char*)ddata;
  auto ncols = [&](int c) { return (size_t)cols - c * cp < cp ? (size_t)cols - c * cp : cp; };
  auto issue = [&](int c) -> int {
    VCPCU_CUDA_TRY(cudaMemcpy2DAsync(stg.buf[c & 1].p, col, dev + c * cp * ld * eb,
                                     (size_t)ld * eb, col, ncols(c), cudaMemcpyDeviceToHost, s));
    VCPCU_CUDA_TRY(cudaEventRecord(stg.ev[c & 1], s));
    return VCPCU_OK;
  };
  if (nchunks > 0 && (st = issue(0))) return st;
  int chunk = 0;
  return save_file(name, type, rows, cols,
                   [&](uint64_t, const unsigned char** p, size_t* n) -> int {
                     const int c = chunk++;
                     VCPCU_CUDA_TRY(cudaEventSynchronize(stg.ev[c & 1]));
                     if (c + 1 < nchunks) {
                       const int si = issue(c + 1);
                       if (si) return si;
                     }
                     *p = (const unsigned char*)stg.buf[c & 1].p;
                     *n = ncols(c) * col;
                     return VCPCU_OK;
                   });
}

extern "C" int vcpcu_vcpmat_load_dev(const char* name, int type, int rows, int cols, void* ddata,
                                     int ld, void* stream) {
  clear_error();
  int st = check_args(name, type, rows, cols);
  if (st) return st;
  if (rows > 0 && (!ddata || ld < rows)) {
    set_error("vcpmat: null data or ld < rows");
    return VCPCU_ERR_INVALID_ARG;
  }
  if ((st = check_device())) return st;
  cudaStream_t s = (cudaStream_t)stream;
  File in;
  std::string file;
  uint64_t crc = 0;
  if ((st = open_for_load(name, type, rows, cols, in, file, crc))) return st;
  const size_t eb = elem_bytes(type), col = (size_t)rows * eb;
  if (col == 0) return read_trailer(in.f, file, crc);
  Staging stg;
  if ((st = stg.init(col))) return st;
  const size_t cp = stg.cols_per;
  unsigned char* dev = (unsigned char*)ddata;
  int b = 0;
  for (size_t c0 = 0; c0 < (size_t)cols; c0 += cp, b ^= 1) {
    const size_t nc = (size_t)cols - c0 < cp ? (size_t)cols - c0 : cp;
    if (c0 >= 2 * cp) VCPCU_CUDA_TRY(cudaEventSynchronize(stg.ev[b]));  // buffer b free
    const size_t n = nc * col;
    if (std::fread(stg.buf[b].p, 1, n, in.f) != n)
      return io_fail("vcpmat: truncated payload in %s", file);
    crc_update(crc, (const unsigned char*)stg.buf[b].p, n);
    VCPCU_CUDA_TRY(cudaMemcpy2DAsync(dev + c0 * ld * eb, (size_t)ld * eb, stg.buf[b].p, col, col,
                                     nc, cudaMemcpyHostToDevice, s));
    VCPCU_CUDA_TRY(cudaEventRecord(stg.ev[b], s));
  }
  VCPCU_CUDA_TRY(cudaStreamSynchronize(s));
  return read_trailer(in.f, file, crc);
}
