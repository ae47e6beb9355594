// les_io.cpp -- the reference's result and restart files, written from the device state
// and read back into it.
//
// Files (gfortran unformatted sequential; one Fortran record per write statement, each
// 3-D record the box (1:im,1:jm,1:km) with i fastest, then j, then k):
//   data20             press.f95:205-216  u, v, w, p, usum, vsum, wsum
//   data21             adam.f95:20-27     fold, gold, hold, fghold
//   data30NNNNNN.dat   anime.f95:370-490  (n, time), then u, v, w, p, usum, vsum, wsum
//   data31NNNNNN.dat   anime.f95:492-595  f, g, h, fold, gold, hold
//   data10             aveflow.f95:209-263  aveu, avew, avev       (the time averages at
//   data11             aveflow.f95:273-344  aveuu, aveww, avevv, uwfx    n == nmax)
// and the restart reader of ifdata.f95:252-480, which reads data30 and data31 back into
// the interiors of those 13 fields (halos stay as they were).  On one process the
// reference's ipmax x jpmax x km box of data30/data31 is im x jm x km.
//
// fghold is declared in the main program (main.f95:122, 133) and never assigned; as a
// main-program array it lives in static storage, which starts zeroed, so data21's fourth
// record is zeros.
//
// Record layout (gfortran's documented form of unformatted sequential files): a record
// is one or more subrecords, each a 4-byte length marker, the data and the marker again.
// A subrecord holds at most 2147483639 bytes; a longer record is split and the leading
// marker of every subrecord but the last is negated (another one follows), the trailing
// marker of every subrecord but the first negated (one precedes).  The split falls on a
// byte count, not on a value.  LES_IO_MAX_SUBRECORD in the environment lowers the limit,
// as gfortran's -fmax-subrecord-length does.  The reference is compiled with
// -fconvert=big-endian (SConstruct:77), so markers and values are big-endian unless the
// caller passes LES_IO_LITTLE_ENDIAN.  The reader takes either order, from the first
// record's markers.
#include <cerrno>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "les_io.h"

namespace {

constexpr uint64_t kMaxSubrecord = 2147483639ull;

uint64_t max_subrecord() {
  const char *e = std::getenv("LES_IO_MAX_SUBRECORD");
  if (e && *e) {
    const long long v = std::atoll(e);
    if (v >= 1 && (uint64_t)v <= kMaxSubrecord) return (uint64_t)v;
  }
  return kMaxSubrecord;
}

bool host_is_big_endian() {
  const uint32_t one = 1;
  unsigned char b[4];
  std::memcpy(b, &one, 4);
  return b[0] == 0;
}

uint32_t bswap32(uint32_t x) {
  return (x >> 24) | ((x >> 8) & 0xff00u) | ((x << 8) & 0xff0000u) | (x << 24);
}

// Puts n 4-byte words in file order (or back in host order: the swap is its own inverse).
void to_order(void *p, size_t n, bool big_endian) {
  if (big_endian == host_is_big_endian()) return;
  uint32_t *w = static_cast<uint32_t *>(p);
  for (size_t q = 0; q < n; ++q) w[q] = bswap32(w[q]);
}

struct File {
  FILE *f = nullptr;
  std::string path;
  ~File() {
    if (f) std::fclose(f);
  }
};

// ---------------------------------------------------------------------------- writer
struct Writer {
  File file;
  bool be = true;
  uint64_t maxsub = kMaxSubrecord;

  bool marker(int32_t v) {
    uint32_t u;
    std::memcpy(&u, &v, 4);
    to_order(&u, 1, be);
    return std::fwrite(&u, 4, 1, file.f) == 1;
  }
  // One record of nbytes bytes already in file order.
  bool record(const void *data, uint64_t nbytes) {
    const char *c = static_cast<const char *>(data);
    uint64_t off = 0;
    bool first = true;
    do {
      const uint64_t len = nbytes - off < maxsub ? nbytes - off : maxsub;
      const bool last = off + len == nbytes;
      if (!marker(last ? (int32_t)len : -(int32_t)len)) return false;
      if (len && std::fwrite(c + off, 1, len, file.f) != len) return false;
      if (!marker(first ? (int32_t)len : -(int32_t)len)) return false;
      off += len;
      first = false;
    } while (off < nbytes);
    return true;
  }
};

int open_writer(les_handle *h, Writer *w, const char *path, int flags) {
  if (!path || !*path) return les_handle_fail(h, LES_ERR_ARG, "file path is empty");
  if (flags & ~LES_IO_LITTLE_ENDIAN) return les_handle_fail(h, LES_ERR_ARG, "unknown file flags");
  w->be = !(flags & LES_IO_LITTLE_ENDIAN);
  w->maxsub = max_subrecord();
  w->file.path = path;
  w->file.f = std::fopen(path, "wb");  // status='replace' / 'unknown': the file is rewritten
  if (!w->file.f)
    return les_handle_fail(h, LES_ERR_IO, (std::string("cannot open ") + path + ": " + std::strerror(errno)).c_str());
  return LES_OK;
}

int write_fail(les_handle *h, const Writer &w) {
  return les_handle_fail(h, LES_ERR_IO, ("write to " + w.file.path + " failed: " + std::strerror(errno)).c_str());
}

// Writes the interior box of each field as one record.  Two host buffers: the device
// copy of the next field runs while the current one is converted and written.
int write_fields(les_handle *h, Writer *w, const int *fields, int nfields) {
  int im, jm, km;
  les_handle_dims(h, &im, &jm, &km);
  const size_t n = (size_t)im * jm * km;
  const int lb[3] = {1, 1, 1}, ub[3] = {im, jm, km};
  std::vector<float> buf[2];
  long long ticket[2] = {-1, -1};
  auto issue = [&](int q) -> int {
    if (fields[q] == 0) return LES_OK;  // a record of zeros (fghold)
    buf[q & 1].resize(n);
    return les_gpu_download_async(h, fields[q], buf[q & 1].data(), lb, ub, &ticket[q & 1]);
  };
  int rc = issue(0);
  for (int q = 0; q < nfields && rc == LES_OK; ++q) {
    std::vector<float> &b = buf[q & 1];
    if (fields[q] == 0) {
      b.assign(n, 0.f);
    } else {
      rc = les_gpu_download_wait(h, ticket[q & 1]);
      ticket[q & 1] = -1;
      if (rc) break;
    }
    if (q + 1 < nfields) {
      rc = issue(q + 1);
      if (rc) break;
    }
    to_order(b.data(), n, w->be);
    if (!w->record(b.data(), (uint64_t)n * 4)) return write_fail(h, *w);
  }
  if (rc) {
    // let copies still in flight land before their buffers go away
    for (int s = 0; s < 2; ++s)
      if (ticket[s] >= 0) les_gpu_download_wait(h, ticket[s]);
    return rc;
  }
  if (std::fflush(w->file.f) != 0) return write_fail(h, *w);
  return LES_OK;
}

int close_writer(les_handle *h, Writer *w) {
  FILE *f = w->file.f;
  w->file.f = nullptr;
  if (std::fclose(f) != 0) return write_fail(h, *w);
  return LES_OK;
}

const int kData20[] = {LES_FIELD_U, LES_FIELD_V, LES_FIELD_W, LES_FIELD_P,
                       LES_FIELD_USUM, LES_FIELD_VSUM, LES_FIELD_WSUM};
const int kData21[] = {LES_FIELD_FOLD, LES_FIELD_GOLD, LES_FIELD_HOLD, 0 /* fghold */};
const int kData31[] = {LES_FIELD_F, LES_FIELD_G, LES_FIELD_H,
                       LES_FIELD_FOLD, LES_FIELD_GOLD, LES_FIELD_HOLD};
const int kData10[] = {LES_FIELD_AVEU, LES_FIELD_AVEW, LES_FIELD_AVEV};
const int kData11[] = {LES_FIELD_AVEUU, LES_FIELD_AVEWW, LES_FIELD_AVEVV, LES_FIELD_UWFX};

int write_file(les_handle *h, const char *path, int flags, const int *fields, int nfields,
               const int *head_n, const float *head_time) {
  Writer w;
  int rc = open_writer(h, &w, path, flags);
  if (rc) return rc;
  if (head_n) {  // write(30) n,time
    uint32_t rec[2];
    std::memcpy(&rec[0], head_n, 4);
    std::memcpy(&rec[1], head_time, 4);
    to_order(rec, 2, w.be);
    if (!w.record(rec, 8)) return write_fail(h, w);
  }
  rc = write_fields(h, &w, fields, nfields);
  if (rc) return rc;
  return close_writer(h, &w);
}

// ---------------------------------------------------------------------------- reader
struct Reader {
  File file;
  bool be = true;
  long long size = 0;
  int nrec = 0;

  bool marker(int32_t *v) {
    uint32_t u;
    if (std::fread(&u, 4, 1, file.f) != 1) return false;
    to_order(&u, 1, be);
    std::memcpy(v, &u, 4);
    return true;
  }
};

// The byte order whose first record's markers agree: leading and trailing length equal,
// the record inside the file.  Big-endian first (the reference's build).
int detect_order(les_handle *h, Reader *r) {
  unsigned char lead[4];
  if (r->size < 8 || std::fread(lead, 1, 4, r->file.f) != 4)
    return les_handle_fail(h, LES_ERR_IO, (r->file.path + ": too short for a Fortran record").c_str());
  for (int order = 0; order < 2; ++order) {
    const bool be = order == 0;
    uint32_t u;
    std::memcpy(&u, lead, 4);
    to_order(&u, 1, be);
    int32_t v;
    std::memcpy(&v, &u, 4);
    const long long len = v < 0 ? -(long long)v : (long long)v;
    if (8 + len > r->size) continue;
    if (std::fseek(r->file.f, (long)(4 + len), SEEK_SET) != 0) continue;
    unsigned char trail[4];
    if (std::fread(trail, 1, 4, r->file.f) != 4) continue;
    uint32_t t;
    std::memcpy(&t, trail, 4);
    to_order(&t, 1, be);
    int32_t tv;
    std::memcpy(&tv, &t, 4);
    if (tv == (int32_t)len) {  // the first subrecord's trailing marker is positive
      r->be = be;
      std::fseek(r->file.f, 0, SEEK_SET);
      return LES_OK;
    }
  }
  return les_handle_fail(h, LES_ERR_IO,
                         (r->file.path + ": not a Fortran unformatted sequential file (record markers do not match)").c_str());
}

int open_reader(les_handle *h, Reader *r, const char *path) {
  if (!path || !*path) return les_handle_fail(h, LES_ERR_ARG, "file path is empty");
  r->file.path = path;
  r->file.f = std::fopen(path, "rb");
  if (!r->file.f)
    return les_handle_fail(h, LES_ERR_IO, (std::string("cannot open ") + path + ": " + std::strerror(errno)).c_str());
  std::fseek(r->file.f, 0, SEEK_END);
  r->size = std::ftell(r->file.f);
  std::fseek(r->file.f, 0, SEEK_SET);
  return detect_order(h, r);
}

// Reads the next record; the first nbytes of it land in dst (file order).  A Fortran
// read of fewer values than the record holds skips the rest; one of more is an error.
int read_record(les_handle *h, Reader *r, void *dst, uint64_t nbytes) {
  char *c = static_cast<char *>(dst);
  uint64_t got = 0;
  const int rec = ++r->nrec;
  auto bad = [&](const std::string &why) {
    return les_handle_fail(h, LES_ERR_IO, (r->file.path + ": record " + std::to_string(rec) + ": " + why).c_str());
  };
  for (bool first = true;; first = false) {
    int32_t lead, trail;
    if (!r->marker(&lead)) return bad("ends before the record");
    const uint64_t len = lead < 0 ? (uint64_t)(-(int64_t)lead) : (uint64_t)lead;
    const uint64_t take = got < nbytes ? (nbytes - got < len ? nbytes - got : len) : 0;
    if (take && std::fread(c + got, 1, take, r->file.f) != take) return bad("data cut short");
    if (len > take && std::fseek(r->file.f, (long)(len - take), SEEK_CUR) != 0) return bad("data cut short");
    got += take;
    if (!r->marker(&trail)) return bad("trailing marker missing");
    const uint64_t tlen = trail < 0 ? (uint64_t)(-(int64_t)trail) : (uint64_t)trail;
    if (tlen != len || (trail < 0) == first) return bad("leading and trailing markers disagree");
    if (lead >= 0) break;
  }
  if (got < nbytes)
    return bad("holds fewer values than the reference reads (" + std::to_string(nbytes / 4) +
               "): was it written for another im x jm x km?");
  return LES_OK;
}

int read_fields(les_handle *h, Reader *r, const int *fields, int nfields) {
  int im, jm, km;
  les_handle_dims(h, &im, &jm, &km);
  const size_t n = (size_t)im * jm * km;
  const int lb[3] = {1, 1, 1}, ub[3] = {im, jm, km};
  std::vector<float> b(n);
  for (int q = 0; q < nfields; ++q) {
    int rc = read_record(h, r, b.data(), (uint64_t)n * 4);
    if (rc) return rc;
    to_order(b.data(), n, r->be);
    rc = les_gpu_upload(h, fields[q], b.data(), lb, ub);
    if (!rc) rc = les_gpu_sync(h);  // b is refilled next
    if (rc) return rc;
  }
  return LES_OK;
}

}  // namespace

extern "C" int les_gpu_write_data20(les_handle *h, const char *path, int flags) {
  if (!h) return LES_ERR_ARG;
  return write_file(h, path, flags, kData20, 7, nullptr, nullptr);
}

extern "C" int les_gpu_write_data21(les_handle *h, const char *path, int flags) {
  if (!h) return LES_ERR_ARG;
  return write_file(h, path, flags, kData21, 4, nullptr, nullptr);
}

extern "C" int les_gpu_write_data30(les_handle *h, const char *path, int n, float time, int flags) {
  if (!h) return LES_ERR_ARG;
  return write_file(h, path, flags, kData20, 7, &n, &time);
}

extern "C" int les_gpu_write_data31(les_handle *h, const char *path, int flags) {
  if (!h) return LES_ERR_ARG;
  return write_file(h, path, flags, kData31, 6, nullptr, nullptr);
}

extern "C" int les_gpu_write_data10(les_handle *h, const char *path, int flags) {
  if (!h) return LES_ERR_ARG;
  return write_file(h, path, flags, kData10, 3, nullptr, nullptr);
}

extern "C" int les_gpu_write_data11(les_handle *h, const char *path, int flags) {
  if (!h) return LES_ERR_ARG;
  return write_file(h, path, flags, kData11, 4, nullptr, nullptr);
}

extern "C" int les_gpu_ifdata_out(les_handle *h, const char *dir, int n, int n1, int nmax, float time, int flags,
                                  int *written) {
  if (!h || !dir) return LES_ERR_ARG;
  if (written) *written = 0;
  if (!(n == n1 - 1 || n == nmax)) return LES_OK;  // anime.f95:370
  if (n < 0 || n > 999999) return les_handle_fail(h, LES_ERR_ARG, "ifdata_out: n does not fit the i6.6 file name");
  std::string base(dir);
  if (base.empty()) base = ".";
  if (base.back() != '/') base += '/';
  char name[32];
  std::snprintf(name, sizeof name, "data30%06d.dat", n);  // anime.f95:375
  int rc = les_gpu_write_data30(h, (base + name).c_str(), n, time, flags);
  if (rc) return rc;
  std::snprintf(name, sizeof name, "data31%06d.dat", n);  // anime.f95:492
  rc = les_gpu_write_data31(h, (base + name).c_str(), flags);
  if (rc) return rc;
  if (written) *written = 1;
  return LES_OK;
}

extern "C" int les_gpu_read_restart(les_handle *h, const char *data30, const char *data31, int *n, float *time) {
  if (!h || !n || !time) return LES_ERR_ARG;
  int head_n;
  float head_time;
  {
    Reader r;
    int rc = open_reader(h, &r, data30);
    if (rc) return rc;
    uint32_t rec[2];
    rc = read_record(h, &r, rec, 8);  // read(30) n,time
    if (rc) return rc;
    to_order(rec, 2, r.be);
    std::memcpy(&head_n, &rec[0], 4);
    std::memcpy(&head_time, &rec[1], 4);
    rc = read_fields(h, &r, kData20, 7);
    if (rc) return rc;
  }
  {
    Reader r;
    int rc = open_reader(h, &r, data31);
    if (rc) return rc;
    rc = read_fields(h, &r, kData31, 6);
    if (rc) return rc;
  }
  *n = head_n;
  *time = head_time;
  return LES_OK;
}
