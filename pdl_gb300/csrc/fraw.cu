// fraw.cu -- PDL::IO::FastRaw files (lib/PDL/IO/FastRaw.pm) read straight
// into an ndarray's memory, host or device, and written from it.
//
// The format: a binary file holding the ndarray's data as laid out in
// memory (dim 0 fastest) and an ASCII header, by default "<name>.hdr":
//   <type id>\n<ndims>\n<dim0> <dim1> ...\n
// (_read_frawhdr / _writefrawhdr, FastRaw.pm:202-230).  A device-resident
// read maps the file and copies the mapping to the device in 64 MiB pieces
// (the driver streams mapped pages through its own staging; no copy of the
// file is made in process memory).  Where the file cannot be mapped it is
// streamed through two pinned staging buffers instead: while one buffer's
// bytes are copied to the device, the next chunk is read into the other.
#include "args.cuh"

#include <fcntl.h>
#include <sys/mman.h>
#include <sys/stat.h>
#include <unistd.h>

#include <cerrno>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <algorithm>
#include <vector>

namespace pg {
namespace {

constexpr size_t FRAW_CHUNK = (size_t)32 << 20, FRAW_MAP_PIECE = (size_t)64 << 20;
// element sizes in PDL's type order (sbyte .. double)
constexpr size_t FSIZE[] = {1, 1, 2, 2, 4, 4, 8, 8, 8, 4, 8};

std::string header_name(const char *name, const char *header) {
  if (header && *header) return header;
  return std::string(name) + ".hdr";
}

bool read_line(FILE *f, std::string &out) {
  out.clear();
  int c;
  bool any = false;
  while ((c = fgetc(f)) != EOF) {
    any = true;
    if (c == '\n') break;
    out.push_back((char)c);
  }
  return any;
}

// two pinned buffers and their events, per device, made on first use; a
// staged transfer holds `use` from its first refill to its last copy, so
// host threads reading or writing files on one device take turns
struct Staging {
  void *buf[2] = {nullptr, nullptr};
  cudaEvent_t ev[2] = {nullptr, nullptr};
  std::mutex use;
};
std::mutex g_stage_mu;
Staging g_stage[64];

pdlgb300_error staging(Staging **out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64)
    return pgh::err(PDLGB300_EFATAL, "no current CUDA device");
  std::lock_guard<std::mutex> lk(g_stage_mu);
  Staging &s = g_stage[dev];
  for (int i = 0; i < 2; i++) {
    if (!s.buf[i] && cudaHostAlloc(&s.buf[i], FRAW_CHUNK, cudaHostAllocDefault) != cudaSuccess) {
      s.buf[i] = nullptr;
      return pgh::err(PDLGB300_EFATAL, "pinned staging allocation failed");
    }
    if (!s.ev[i] && cudaEventCreateWithFlags(&s.ev[i], cudaEventDisableTiming) != cudaSuccess) {
      s.ev[i] = nullptr;
      return pgh::err(PDLGB300_EFATAL, "event creation failed");
    }
  }
  *out = &s;
  return pgh::ok();
}

}  // namespace
}  // namespace pg

using namespace pg;

extern "C" {

pdlgb300_error pdlgb300_fraw_header(const char *name, const char *header, pdlgb300_ndarray *x) {
  if (!name || !x) return pgh::err(PDLGB300_EUSERERROR, "fraw: NULL argument");
  const std::string h = header_name(name, header);
  FILE *f = fopen(h.c_str(), "r");
  if (!f)
    return pgh::err(PDLGB300_EUSERERROR, "Couldn't open '%s' for reading: %s", h.c_str(),
                    strerror(errno));
  std::string tid, nd, dims;
  const bool ok1 = read_line(f, tid), ok2 = read_line(f, nd), ok3 = read_line(f, dims);
  fclose(f);
  (void)ok1;
  (void)ok2;
  if (!ok3) return pgh::err(PDLGB300_EUSERERROR, "Format error in '%s'", h.c_str());
  char *end = nullptr;
  const long t = strtol(tid.c_str(), &end, 10);
  if (end == tid.c_str() || t < 0 || t >= PDLGB300_NTYPES)
    return pgh::err(PDLGB300_EUSERERROR, "fraw header '%s': unknown type '%s'", h.c_str(), tid.c_str());
  if (t > PDLGB300_D)
    return pgh::err(PDLGB300_EUSERERROR, "fraw header '%s': type %ld is not on this path", h.c_str(), t);
  const long ndims = strtol(nd.c_str(), nullptr, 10);
  std::vector<long long> d;
  const char *p = dims.c_str();
  for (;;) {
    while (*p == ' ' || *p == '\t' || *p == '\r') p++;
    if (!*p) break;
    char *e2 = nullptr;
    const long long v = strtoll(p, &e2, 10);
    if (e2 == p) break;
    d.push_back(v);
    p = e2;
  }
  if ((long)d.size() != ndims || ndims > PDLGB300_MAXDIMS)
    return pgh::err(PDLGB300_EUSERERROR, "Format error reading fraw header file '%s'", h.c_str());
  for (long long v : d)
    if (v < 0) return pgh::err(PDLGB300_EUSERERROR, "Format error reading fraw header file '%s'", h.c_str());
  x->datatype = (int32_t)t;
  x->ndims = (int32_t)ndims;
  int64_t s = 1;
  for (int i = 0; i < (int)ndims; i++) {
    x->dims[i] = d[i];
    x->incs[i] = s;
    s *= d[i];
  }
  x->offs = 0;
  x->state &= ~PDLGB300_NOMYDIMS;
  return pgh::ok();
}

pdlgb300_error pdlgb300_readfraw_into(const char *name, pdlgb300_ndarray *x) {
  if (!name || !x) return pgh::err(PDLGB300_EUSERERROR, "fraw: NULL argument");
  if (x->datatype < 0 || x->datatype > PDLGB300_D)
    return pgh::err(PDLGB300_EUSERERROR, "readfraw: type %d is not on this path", x->datatype);
  int64_t n = 1;
  for (int i = 0; i < x->ndims; i++) n *= x->dims[i];
  const size_t len = (size_t)n * FSIZE[x->datatype];
  FILE *f = fopen(name, "rb");
  if (!f)
    return pgh::err(PDLGB300_EUSERERROR, "Couldn't open '%s' for reading: %s", name, strerror(errno));
  pdlgb300_error e = pgh::ok();
  size_t got = 0;
  if (!x->ddata) {
    // host memory: read in place; a short file leaves the rest zero, as the
    // reference's readfraw (it reads into zeroes())
    char *dst = (char *)x->data;
    if (!dst && len) e = pgh::err(PDLGB300_EUSERERROR, "readfraw: ndarray has no memory");
    while (!e.error && got < len) {
      const size_t r = fread(dst + got, 1, len - got, f);
      if (r == 0) break;
      got += r;
    }
    if (!e.error && got < len) memset(dst + got, 0, len - got);
    fclose(f);
    return e;
  }
  {
    // the mapped file, copied in pieces
    struct stat st;
    const int fd = fileno(f);
    if (fstat(fd, &st) == 0 && st.st_size > 0 && len > 0) {
      const size_t avail = std::min(len, (size_t)st.st_size);
      void *map = mmap(nullptr, avail, PROT_READ, MAP_PRIVATE, fd, 0);
      if (map != MAP_FAILED) {
        madvise(map, avail, MADV_SEQUENTIAL);
        char *dst = (char *)x->ddata;
        cudaError_t ce = cudaSuccess;
        for (size_t off = 0; off < avail && ce == cudaSuccess; off += FRAW_MAP_PIECE)
          ce = cudaMemcpyAsync(dst + off, (const char *)map + off,
                               std::min(FRAW_MAP_PIECE, avail - off), cudaMemcpyHostToDevice,
                               pgh::stream());
        if (ce == cudaSuccess && avail < len)
          ce = cudaMemsetAsync(dst + avail, 0, len - avail, pgh::stream());
        if (ce == cudaSuccess) ce = cudaStreamSynchronize(pgh::stream());
        munmap(map, avail);
        fclose(f);
        if (ce != cudaSuccess) return pgh::err(PDLGB300_EFATAL, "readfraw: %s", cudaGetErrorString(ce));
        return pgh::ok();
      }
    }
  }
  Staging *s = nullptr;
  e = staging(&s);
  if (e.error) {
    fclose(f);
    return e;
  }
  std::lock_guard<std::mutex> turn(s->use);
  char *dst = (char *)x->ddata;
  int k = 0;
  while (!e.error && got < len) {
    // wait for this buffer's previous copy, refill it, copy it on
    if (cudaEventSynchronize(s->ev[k]) != cudaSuccess) {
      e = pgh::err(PDLGB300_EFATAL, "readfraw: %s", cudaGetErrorString(cudaGetLastError()));
      break;
    }
    const size_t want = std::min(FRAW_CHUNK, len - got);
    const size_t r = fread(s->buf[k], 1, want, f);
    if (r == 0) break;
    cudaError_t ce = cudaMemcpyAsync(dst + got, s->buf[k], r, cudaMemcpyHostToDevice, pgh::stream());
    if (ce == cudaSuccess) ce = cudaEventRecord(s->ev[k], pgh::stream());
    if (ce != cudaSuccess) e = pgh::err(PDLGB300_EFATAL, "readfraw: %s", cudaGetErrorString(ce));
    got += r;
    k ^= 1;
  }
  fclose(f);
  if (!e.error && got < len) {
    cudaError_t ce = cudaMemsetAsync(dst + got, 0, len - got, pgh::stream());
    if (ce != cudaSuccess) e = pgh::err(PDLGB300_EFATAL, "readfraw: %s", cudaGetErrorString(ce));
  }
  if (!e.error) {
    cudaError_t ce = cudaStreamSynchronize(pgh::stream());
    if (ce != cudaSuccess) e = pgh::err(PDLGB300_EFATAL, "readfraw: %s", cudaGetErrorString(ce));
  }
  return e;
}

pdlgb300_error pdlgb300_writefraw(const pdlgb300_ndarray *x, const char *name, const char *header) {
  if (!name || !x) return pgh::err(PDLGB300_EUSERERROR, "fraw: NULL argument");
  if (x->datatype < 0 || x->datatype > PDLGB300_D)
    return pgh::err(PDLGB300_EUSERERROR, "writefraw: type %d is not on this path", x->datatype);
  // the data as laid out in memory: a contiguous ndarray
  int64_t n = 1, s = 1;
  for (int i = 0; i < x->ndims; i++) {
    if (x->dims[i] > 1 && x->incs[i] != s)
      return pgh::err(PDLGB300_EUSERERROR, "writefraw: the ndarray must be contiguous");
    s *= x->dims[i];
    n *= x->dims[i];
  }
  const std::string h = header_name(name, header);
  FILE *fh = fopen(h.c_str(), "w");
  if (!fh)
    return pgh::err(PDLGB300_EUSERERROR, "Couldn't open '%s' for writing: %s", h.c_str(),
                    strerror(errno));
  fprintf(fh, "%d\n%d\n", x->datatype, x->ndims);
  for (int i = 0; i < x->ndims; i++) fprintf(fh, i ? " %lld" : "%lld", (long long)x->dims[i]);
  fprintf(fh, "\n");
  fclose(fh);
  FILE *f = fopen(name, "wb");
  if (!f)
    return pgh::err(PDLGB300_EUSERERROR, "Couldn't open '%s' for writing: %s", name, strerror(errno));
  const size_t ts = FSIZE[x->datatype];
  const size_t len = (size_t)n * ts;
  pdlgb300_error e = pgh::ok();
  if (!x->ddata) {
    const char *src = (const char *)x->data + x->offs * (int64_t)ts;
    if (len && fwrite(src, 1, len, f) != len) e = pgh::err(PDLGB300_EFATAL, "writefraw: short write");
    fclose(f);
    return e;
  }
  Staging *st = nullptr;
  e = staging(&st);
  if (e.error) {
    fclose(f);
    return e;
  }
  std::lock_guard<std::mutex> turn(st->use);
  const char *src = (const char *)x->ddata + x->offs * (int64_t)ts;
  size_t done = 0;
  while (!e.error && done < len) {
    const size_t want = std::min(FRAW_CHUNK, len - done);
    cudaError_t ce = cudaMemcpyAsync(st->buf[0], src + done, want, cudaMemcpyDeviceToHost, pgh::stream());
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(pgh::stream());
    if (ce != cudaSuccess) {
      e = pgh::err(PDLGB300_EFATAL, "writefraw: %s", cudaGetErrorString(ce));
      break;
    }
    if (fwrite(st->buf[0], 1, want, f) != want) e = pgh::err(PDLGB300_EFATAL, "writefraw: short write");
    done += want;
  }
  fclose(f);
  return e;
}

}  // extern "C"
