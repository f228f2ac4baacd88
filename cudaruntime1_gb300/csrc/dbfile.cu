// dbfile.cu -- on-disk format of a device-resident database: written once,
// loaded straight back into HBM for serving (no summary rebuild).
//
// Layout (little-endian, 8-byte aligned sections):
//   header  64 B : magic "TSIMDB\0\1", version, segments per candidate,
//                  count, total points, longest trajectory, reserved
//   off     int64[count + 1]            CSR offsets (off[0] = 0, increasing)
//   pts     float2[total]               points (x, y), the reference's Point
//   box     float4[count]               bounding boxes (x0, y0, x1, y1)
//   ends    float4[count]               first and last point
//   len     int32[count], padded to 8 B
//   segbox  float4[count * segments]    boxes of the candidate's column segments
//   segsum  float2[count * segments]    sums of the points of those segments
//   sum     uint64                      checksum of everything before it
// The reference keeps no database on disk (its inputs are generated per run).
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "tsim_internal.cuh"

namespace tsim {
namespace {

constexpr char kMagic[8] = {'T', 'S', 'I', 'M', 'D', 'B', 0, 1};
constexpr uint32_t kVersion = 2;
constexpr size_t kChunkBytes = size_t(64) << 20;  // staging per transfer

struct Header {
  char magic[8];
  uint32_t version;
  uint32_t segs;
  int64_t count;
  int64_t total;
  int64_t max_len;
  uint64_t reserved[3];
};
static_assert(sizeof(Header) == 64, "header is 64 bytes");

// 64-bit word mix (multiply-xorshift per word, then a final avalanche)
struct Sum {
  uint64_t h = 0x9E3779B97F4A7C15ull;
  uint64_t tail = 0;
  int ntail = 0;
  void add(const void* p, size_t n) {
    const unsigned char* b = static_cast<const unsigned char*>(p);
    while (n && ntail) {
      tail |= (uint64_t)*b++ << (8 * ntail);
      --n;
      if (++ntail == 8) {
        word(tail);
        tail = 0;
        ntail = 0;
      }
    }
    while (n >= 8) {
      uint64_t w;
      memcpy(&w, b, 8);
      word(w);
      b += 8;
      n -= 8;
    }
    while (n) {
      tail |= (uint64_t)*b++ << (8 * ntail++);
      --n;
    }
  }
  void word(uint64_t w) {
    h ^= w * 0xBF58476D1CE4E5B9ull;
    h = (h << 27 | h >> 37) * 0x94D049BB133111EBull;
  }
  uint64_t value() {
    uint64_t x = h ^ (tail + (uint64_t)ntail);
    x ^= x >> 31;
    x *= 0xD6E8FEB86659FD93ull;
    x ^= x >> 32;
    return x;
  }
};

struct File {
  FILE* f = nullptr;
  ~File() {
    if (f) fclose(f);
  }
};

// device -> file through a host buffer, chunk by chunk
int write_dev(FILE* f, Sum& s, const void* dev, size_t bytes, std::vector<char>& buf) {
  const char* d = static_cast<const char*>(dev);
  for (size_t o = 0; o < bytes; o += buf.size()) {
    const size_t n = std::min(buf.size(), bytes - o);
    TSIM_CUDA(cudaMemcpy(buf.data(), d + o, n, cudaMemcpyDeviceToHost));
    s.add(buf.data(), n);
    if (fwrite(buf.data(), 1, n, f) != n) return fail(TSIM_ERR_INVALID_ARG, "short write");
  }
  return TSIM_OK;
}

int write_host(FILE* f, Sum& s, const void* p, size_t bytes) {
  s.add(p, bytes);
  if (bytes && fwrite(p, 1, bytes, f) != bytes) return fail(TSIM_ERR_INVALID_ARG, "short write");
  return TSIM_OK;
}

// file -> device through pinned staging, chunk by chunk
int read_dev(FILE* f, Sum& s, void* dev, size_t bytes, char* pinned, cudaStream_t st) {
  char* d = static_cast<char*>(dev);
  for (size_t o = 0; o < bytes; o += kChunkBytes) {
    const size_t n = std::min(kChunkBytes, bytes - o);
    TSIM_CUDA(cudaStreamSynchronize(st));  // the staging buffer is free again
    if (fread(pinned, 1, n, f) != n) return fail(TSIM_ERR_INVALID_ARG, "database file is truncated");
    s.add(pinned, n);
    TSIM_CUDA(cudaMemcpyAsync(d + o, pinned, n, cudaMemcpyHostToDevice, st));
  }
  TSIM_CUDA(cudaStreamSynchronize(st));
  return TSIM_OK;
}

int read_host(FILE* f, Sum& s, void* p, size_t bytes) {
  if (bytes && fread(p, 1, bytes, f) != bytes)
    return fail(TSIM_ERR_INVALID_ARG, "database file is truncated");
  s.add(p, bytes);
  return TSIM_OK;
}

size_t pad8(size_t b) { return (b + 7) & ~size_t(7); }

}  // namespace
}  // namespace tsim

using namespace tsim;

extern "C" int tsim_db_save(const tsim_db* db, const char* path) {
  TSIM_CHECK_ARG(db && path, "NULL argument");
  TSIM_CHECK_ARG(db->ctx != nullptr, "database's context was destroyed");
  TSIM_CUDA(cudaSetDevice(db->ctx->device));
  TSIM_CUDA(cudaStreamSynchronize(db->ctx->stream));
  File fh;
  fh.f = fopen(path, "wb");
  if (!fh.f) return fail(TSIM_ERR_INVALID_ARG, std::string("cannot write ") + path);
  Header h{};
  memcpy(h.magic, kMagic, 8);
  h.version = kVersion;
  h.segs = kSegs;
  h.count = db->count;
  h.total = db->total;
  h.max_len = db->max_len;
  if (fwrite(&h, sizeof(h), 1, fh.f) != 1) return fail(TSIM_ERR_INVALID_ARG, "short write");
  Sum s;
  s.add(&h, sizeof(h));
  std::vector<char> buf(kChunkBytes);
  const size_t n = (size_t)db->count;
  TSIM_TRY(write_host(fh.f, s, db->h_off.data(), sizeof(int64_t) * (n + 1)));
  TSIM_TRY(write_dev(fh.f, s, db->pts, sizeof(float2) * (size_t)db->total, buf));
  TSIM_TRY(write_dev(fh.f, s, db->box, sizeof(float4) * n, buf));
  TSIM_TRY(write_dev(fh.f, s, db->ends, sizeof(float4) * n, buf));
  TSIM_TRY(write_dev(fh.f, s, db->len, sizeof(int) * n, buf));
  const char zeros[8] = {0};
  TSIM_TRY(write_host(fh.f, s, zeros, pad8(sizeof(int) * n) - sizeof(int) * n));
  TSIM_TRY(write_dev(fh.f, s, db->segbox, sizeof(float4) * n * kSegs, buf));
  TSIM_TRY(write_dev(fh.f, s, db->segsum, sizeof(float2) * n * kSegs, buf));
  const uint64_t sum = s.value();
  if (fwrite(&sum, 8, 1, fh.f) != 1) return fail(TSIM_ERR_INVALID_ARG, "short write");
  const int rc = fclose(fh.f);
  fh.f = nullptr;
  return rc == 0 ? TSIM_OK : fail(TSIM_ERR_INVALID_ARG, std::string("cannot write ") + path);
}

extern "C" int tsim_db_load(tsim_ctx* ctx, const char* path, tsim_db** out) {
  TSIM_CHECK_ARG(ctx && path && out, "NULL argument");
  *out = nullptr;
  File fh;
  fh.f = fopen(path, "rb");
  if (!fh.f) return fail(TSIM_ERR_INVALID_ARG, std::string("cannot read ") + path);
  Header h{};
  if (fread(&h, sizeof(h), 1, fh.f) != 1 || memcmp(h.magic, kMagic, 8) != 0)
    return fail(TSIM_ERR_INVALID_ARG, "not a tsim database file");
  if (h.version != kVersion) return fail(TSIM_ERR_UNSUPPORTED, "unknown database file version");
  if (h.segs != (uint32_t)kSegs)
    return fail(TSIM_ERR_UNSUPPORTED, "database file has another segment count; rebuild it");
  if (h.count < 0 || h.count > 0x7fffffff || h.total < 0 || h.total > (int64_t(1) << 56) ||
      h.max_len < 0 || h.max_len > 0x7fffffff)
    return fail(TSIM_ERR_INVALID_ARG, "corrupt database header");
  {  // the header's sizes must match the file's before anything is allocated
    const uint64_t c = (uint64_t)h.count;
    const uint64_t want = sizeof(Header) + 8 * (c + 1) + 8 * (uint64_t)h.total + 32 * c +
                          pad8(4 * c) + (16 + 8) * (uint64_t)kSegs * c + 8;
    if (fseeko(fh.f, 0, SEEK_END) != 0) return fail(TSIM_ERR_INVALID_ARG, "cannot seek database file");
    const off_t have = ftello(fh.f);
    if (have < 0 || (uint64_t)have != want || fseeko(fh.f, sizeof(Header), SEEK_SET) != 0)
      return fail(TSIM_ERR_INVALID_ARG, "database file size does not match its header");
  }
  Sum s;
  s.add(&h, sizeof(h));
  const size_t n = (size_t)h.count;
  std::vector<int64_t> off(n + 1);
  TSIM_TRY(read_host(fh.f, s, off.data(), sizeof(int64_t) * (n + 1)));
  int64_t ml = 0;
  if (off[0] != 0 || off[n] != h.total) return fail(TSIM_ERR_INVALID_ARG, "corrupt offsets");
  for (size_t t = 0; t < n; ++t) {
    if (off[t + 1] <= off[t]) return fail(TSIM_ERR_INVALID_ARG, "corrupt offsets");
    ml = std::max<int64_t>(ml, off[t + 1] - off[t]);
  }
  if (ml != h.max_len) return fail(TSIM_ERR_INVALID_ARG, "corrupt header (longest trajectory)");
  TSIM_CUDA(cudaSetDevice(ctx->device));
  tsim_db* db = new tsim_db;
  db->ctx = ctx;
  db->count = (int)n;
  db->total = h.total;
  db->max_len = (int)ml;
  db->owns = true;
  db->h_off = std::move(off);
  char* pinned = nullptr;
  int st = TSIM_OK;
  cudaError_t e = dev_malloc(reinterpret_cast<void**>(&db->pts), sizeof(float2) * std::max<int64_t>(db->total, 1));
  if (e == cudaSuccess) e = dev_malloc(reinterpret_cast<void**>(&db->off), sizeof(int64_t) * (n + 1));
  if (e == cudaSuccess) e = dev_malloc(reinterpret_cast<void**>(&db->segbox), sizeof(float4) * kSegs * std::max<size_t>(n, 1));
  if (e == cudaSuccess) e = dev_malloc(reinterpret_cast<void**>(&db->segsum), sizeof(float2) * kSegs * std::max<size_t>(n, 1));
  if (e == cudaSuccess) e = dev_malloc(reinterpret_cast<void**>(&db->box), sizeof(float4) * std::max<size_t>(n, 1));
  if (e == cudaSuccess) e = dev_malloc(reinterpret_cast<void**>(&db->ends), sizeof(float4) * std::max<size_t>(n, 1));
  if (e == cudaSuccess) e = dev_malloc(reinterpret_cast<void**>(&db->len), sizeof(int) * std::max<size_t>(n, 1));
  if (e == cudaSuccess) e = host_alloc((void**)&pinned, kChunkBytes);
  if (e != cudaSuccess) st = cuda_fail(e, "tsim_db_load allocation", __FILE__, __LINE__);
  if (st == TSIM_OK) {
    e = cudaMemcpyAsync(db->off, db->h_off.data(), sizeof(int64_t) * (n + 1),
                        cudaMemcpyHostToDevice, ctx->stream);
    if (e != cudaSuccess) st = cuda_fail(e, "tsim_db_load offsets", __FILE__, __LINE__);
  }
  char pad[8];
  if (st == TSIM_OK) st = read_dev(fh.f, s, db->pts, sizeof(float2) * (size_t)db->total, pinned, ctx->stream);
  if (st == TSIM_OK) st = read_dev(fh.f, s, db->box, sizeof(float4) * n, pinned, ctx->stream);
  if (st == TSIM_OK) st = read_dev(fh.f, s, db->ends, sizeof(float4) * n, pinned, ctx->stream);
  if (st == TSIM_OK) st = read_dev(fh.f, s, db->len, sizeof(int) * n, pinned, ctx->stream);
  if (st == TSIM_OK) st = read_host(fh.f, s, pad, pad8(sizeof(int) * n) - sizeof(int) * n);
  if (st == TSIM_OK)
    st = read_dev(fh.f, s, db->segbox, sizeof(float4) * n * kSegs, pinned, ctx->stream);
  if (st == TSIM_OK)
    st = read_dev(fh.f, s, db->segsum, sizeof(float2) * n * kSegs, pinned, ctx->stream);
  uint64_t want = 0;
  if (st == TSIM_OK && fread(&want, 8, 1, fh.f) != 1)
    st = fail(TSIM_ERR_INVALID_ARG, "database file is truncated");
  if (st == TSIM_OK && want != s.value())
    st = fail(TSIM_ERR_INVALID_ARG, "database file checksum mismatch");
  if (pinned) cudaFreeHost(pinned);
  if (st != TSIM_OK) {
    cudaStreamSynchronize(ctx->stream);
    cudaFree(db->pts);
    cudaFree(db->off);
    cudaFree(db->box);
    cudaFree(db->ends);
    cudaFree(db->len);
    cudaFree(db->segbox);
    cudaFree(db->segsum);
    delete db;
    return st;
  }
  ctx->dbs.push_back(db);
  *out = db;
  return TSIM_OK;
}
