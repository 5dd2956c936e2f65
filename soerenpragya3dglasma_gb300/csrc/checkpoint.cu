// checkpoint.cu -- configuration files: the reference's text format and a bit-exact binary format.
//
// Text (IO::SaveConfiguration / SaveConfigurationJ, S/IO/SaveConfiguration.cpp:6-93; read back as
// IO::LoadConfiguration does, S/IO/LoadConfiguration.cpp:3-200).  One line per entry, ghost slices
// included (z from -1 to Nz, then y, then x), numbers with 15 significant digits (the reference's
// OUTPUT_PRECISION = digits10 of double, S/Definitions.cpp:33-34, in the stream's default format,
// which is printf's %.15g):
//   links     "x y z mu  re(U_00) im(U_00) ... re(U_22) im(U_22) "   (9 entries in the order i + 3j)
//   E         "x y z mu e^1 ... e^8"
//   currents  "x y z a JpStat^a Jp^a JmStat^a Jm^a "
// Reading checks that the link and field lines come in the writer's order (as the reference
// does) and that every entry is present, and returns a status instead of exiting.  The currents
// file is read for all eight colours (the reference's LoadCurrents loop only fills colours 0-2).
// 15 digits do not pin a double: a text round trip moves values by up to ~5e-16 relative.
//
// Binary (no reference counterpart): a 64-byte header ("GLASMACK", version, Nx, Ny, Nz, spacings)
// followed by U, UOld, E, Jp, Jm, JpStat, JmStat in the reference's host layout (doubles, ghost
// slices included) — a restart file that reproduces the fields bit for bit.
#include <cerrno>
#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/glasma_gb300.h"
#include "handle.h"

namespace {

thread_local std::string g_io_error;
int io_fail(int status, const std::string& m) {
  g_io_error = m;
  return status;
}

struct Dims {
  int nx, ny, nz;
  long long sites() const { return (long long)nx * ny * (nz + 2); }
  long long site(int x, int y, int z) const { return x + (long long)nx * (y + (long long)ny * (z + 1)); }
};

bool dims_ok(int nx, int ny, int nz) { return nx >= 1 && ny >= 1 && nz >= 1; }

// Buffered line writer
struct Writer {
  FILE* f = nullptr;
  std::vector<char> buf;
  size_t used = 0;
  bool ok = true;
  explicit Writer(const char* path) : buf(1 << 20) { f = std::fopen(path, "w"); }
  ~Writer() {
    flush();
    if (f) std::fclose(f);
  }
  void flush() {
    if (f && used) ok = ok && std::fwrite(buf.data(), 1, used, f) == used;
    used = 0;
  }
  void put(const char* fmt, ...) __attribute__((format(printf, 2, 3)));
};
void Writer::put(const char* fmt, ...) {
  if (buf.size() - used < 512) flush();
  va_list ap;
  va_start(ap, fmt);
  const int n = std::vsnprintf(buf.data() + used, buf.size() - used, fmt, ap);
  va_end(ap);
  if (n < 0 || (size_t)n >= buf.size() - used) {
    ok = false;
    return;
  }
  used += (size_t)n;
}

int write_links(const Dims& d, const double* U, const char* path) {
  Writer w(path);
  if (!w.f) return io_fail(GLASMA_ERR_INVALID_ARGUMENT, std::string("cannot open ") + path + " for writing");
  for (int z = -1; z <= d.nz; z++)
    for (int y = 0; y < d.ny; y++)
      for (int x = 0; x < d.nx; x++)
        for (int mu = 0; mu < 3; mu++) {
          const double* u = U + 18 * (3 * d.site(x, y, z) + mu);
          w.put("%d %d %d %d ", x, y, z, mu);
          for (int k = 0; k < 9; k++) w.put("%.15g %.15g ", u[2 * k], u[2 * k + 1]);
          w.put("\n");
        }
  w.flush();
  return w.ok ? GLASMA_OK : io_fail(GLASMA_ERR_INVALID_ARGUMENT, std::string("write failed: ") + path);
}

int write_efield(const Dims& d, const double* E, const char* path) {
  Writer w(path);
  if (!w.f) return io_fail(GLASMA_ERR_INVALID_ARGUMENT, std::string("cannot open ") + path + " for writing");
  for (int z = -1; z <= d.nz; z++)
    for (int y = 0; y < d.ny; y++)
      for (int x = 0; x < d.nx; x++)
        for (int mu = 0; mu < 3; mu++) {
          const double* e = E + 8 * (3 * d.site(x, y, z) + mu);
          w.put("%d %d %d %d", x, y, z, mu);
          for (int a = 0; a < 8; a++) w.put(" %.15g", e[a]);
          w.put("\n");
        }
  w.flush();
  return w.ok ? GLASMA_OK : io_fail(GLASMA_ERR_INVALID_ARGUMENT, std::string("write failed: ") + path);
}

int write_currents(const Dims& d, const double* JpS, const double* Jp, const double* JmS, const double* Jm,
                   const char* path) {
  Writer w(path);
  if (!w.f) return io_fail(GLASMA_ERR_INVALID_ARGUMENT, std::string("cannot open ") + path + " for writing");
  for (int z = -1; z <= d.nz; z++)
    for (int y = 0; y < d.ny; y++)
      for (int x = 0; x < d.nx; x++)
        for (int a = 0; a < 8; a++) {
          const long long i = 8 * d.site(x, y, z) + a;
          w.put("%d %d %d %d %.15g %.15g %.15g %.15g \n", x, y, z, a, JpS[i], Jp[i], JmS[i], Jm[i]);
        }
  w.flush();
  return w.ok ? GLASMA_OK : io_fail(GLASMA_ERR_INVALID_ARGUMENT, std::string("write failed: ") + path);
}

// Line reader: parses ints and doubles with strtol/strtod (correctly rounded, as the reference's
// stream extraction)
struct Reader {
  FILE* f = nullptr;
  std::string path;
  long long line_no = 0;
  std::vector<char> line;
  explicit Reader(const char* p) : path(p), line(1 << 16) { f = std::fopen(p, "r"); }
  ~Reader() {
    if (f) std::fclose(f);
  }
  // next non-empty line into `line`; false at end of file
  bool next() {
    for (;;) {
      if (!std::fgets(line.data(), (int)line.size(), f)) return false;
      line_no++;
      const char* p = line.data();
      while (*p == ' ' || *p == '\t' || *p == '\r') p++;
      if (*p != '\n' && *p != 0) return true;
    }
  }
  std::string where() const { return path + ":" + std::to_string(line_no); }
};

bool parse_ints(char*& p, int* v, int n) {
  for (int i = 0; i < n; i++) {
    char* end = nullptr;
    errno = 0;
    const long x = std::strtol(p, &end, 10);
    if (end == p || errno) return false;
    v[i] = (int)x;
    p = end;
  }
  return true;
}
bool parse_doubles(char*& p, double* v, int n) {
  for (int i = 0; i < n; i++) {
    char* end = nullptr;
    v[i] = std::strtod(p, &end);
    if (end == p) return false;
    p = end;
  }
  return true;
}

int read_links(const Dims& d, double* U, const char* path) {
  Reader r(path);
  if (!r.f) return io_fail(GLASMA_ERR_INVALID_ARGUMENT, std::string("cannot open ") + path);
  for (int z = -1; z <= d.nz; z++)
    for (int y = 0; y < d.ny; y++)
      for (int x = 0; x < d.nx; x++)
        for (int mu = 0; mu < 3; mu++) {
          if (!r.next()) return io_fail(GLASMA_ERR_INVALID_ARGUMENT, r.where() + ": file ends before all links");
          char* p = r.line.data();
          int pos[4];
          if (!parse_ints(p, pos, 4) || pos[0] != x || pos[1] != y || pos[2] != z || pos[3] != mu)
            return io_fail(GLASMA_ERR_INVALID_ARGUMENT, r.where() + ": expected link " + std::to_string(x) + " " +
                                                            std::to_string(y) + " " + std::to_string(z) + " " +
                                                            std::to_string(mu));
          if (!parse_doubles(p, U + 18 * (3 * d.site(x, y, z) + mu), 18))
            return io_fail(GLASMA_ERR_INVALID_ARGUMENT, r.where() + ": 18 numbers expected");
        }
  if (r.next()) return io_fail(GLASMA_ERR_INVALID_ARGUMENT, r.where() + ": more links than the lattice holds");
  return GLASMA_OK;
}

int read_efield(const Dims& d, double* E, const char* path) {
  Reader r(path);
  if (!r.f) return io_fail(GLASMA_ERR_INVALID_ARGUMENT, std::string("cannot open ") + path);
  for (int z = -1; z <= d.nz; z++)
    for (int y = 0; y < d.ny; y++)
      for (int x = 0; x < d.nx; x++)
        for (int mu = 0; mu < 3; mu++) {
          if (!r.next()) return io_fail(GLASMA_ERR_INVALID_ARGUMENT, r.where() + ": file ends before all fields");
          char* p = r.line.data();
          int pos[4];
          if (!parse_ints(p, pos, 4) || pos[0] != x || pos[1] != y || pos[2] != z || pos[3] != mu)
            return io_fail(GLASMA_ERR_INVALID_ARGUMENT, r.where() + ": expected field " + std::to_string(x) + " " +
                                                            std::to_string(y) + " " + std::to_string(z) + " " +
                                                            std::to_string(mu));
          if (!parse_doubles(p, E + 8 * (3 * d.site(x, y, z) + mu), 8))
            return io_fail(GLASMA_ERR_INVALID_ARGUMENT, r.where() + ": 8 colour components expected");
        }
  if (r.next()) return io_fail(GLASMA_ERR_INVALID_ARGUMENT, r.where() + ": more fields than the lattice holds");
  return GLASMA_OK;
}

int read_currents(const Dims& d, double* JpS, double* Jp, double* JmS, double* Jm, const char* path) {
  Reader r(path);
  if (!r.f) return io_fail(GLASMA_ERR_INVALID_ARGUMENT, std::string("cannot open ") + path);
  const long long n = 8 * d.sites();
  std::vector<char> seen((size_t)n, 0);
  long long count = 0;
  while (r.next()) {
    char* p = r.line.data();
    int pos[4];
    double v[4];
    if (!parse_ints(p, pos, 4) || !parse_doubles(p, v, 4))
      return io_fail(GLASMA_ERR_INVALID_ARGUMENT, r.where() + ": x y z a and four numbers expected");
    const int x = pos[0], y = pos[1], z = pos[2], a = pos[3];
    if (x < 0 || x >= d.nx || y < 0 || y >= d.ny || z < -1 || z > d.nz || a < 0 || a > 7)
      return io_fail(GLASMA_ERR_INVALID_ARGUMENT, r.where() + ": position outside the lattice");
    const long long i = 8 * d.site(x, y, z) + a;
    JpS[i] = v[0];
    Jp[i] = v[1];
    JmS[i] = v[2];
    Jm[i] = v[3];
    if (!seen[(size_t)i]) {
      seen[(size_t)i] = 1;
      count++;
    }
  }
  if (count != n)
    return io_fail(GLASMA_ERR_INVALID_ARGUMENT, std::string(path) + ": " + std::to_string(n - count) +
                                                    " current entries missing");
  return GLASMA_OK;
}

// ---- binary
constexpr char kMagic[8] = {'G', 'L', 'A', 'S', 'M', 'A', 'C', 'K'};
struct BinHeader {
  char magic[8];
  int32_t version, nx, ny, nz;
  double a[3];
  int64_t steps_done;
  int64_t reserved;
};
static_assert(sizeof(BinHeader) == 64, "header is 64 bytes");
constexpr int kBinFields[7] = {GLASMA_FIELD_U,  GLASMA_FIELD_UOLD,   GLASMA_FIELD_E,     GLASMA_FIELD_JP,
                               GLASMA_FIELD_JM, GLASMA_FIELD_JPSTAT, GLASMA_FIELD_JMSTAT};

}  // namespace

extern "C" {

const char* glasma_io_last_error(void) { return g_io_error.c_str(); }

int glasma_write_text_host(int nx, int ny, int nz, const double* U, const double* E, const double* JpStat,
                           const double* Jp, const double* JmStat, const double* Jm, const char* u_path,
                           const char* e_path, const char* j_path) {
  if (!dims_ok(nx, ny, nz)) return io_fail(GLASMA_ERR_BAD_SHAPE, "bad lattice shape");
  const Dims d{nx, ny, nz};
  int st = GLASMA_OK;
  if (u_path) {
    if (!U) return io_fail(GLASMA_ERR_INVALID_ARGUMENT, "links path given without links");
    if ((st = write_links(d, U, u_path))) return st;
  }
  if (e_path) {
    if (!E) return io_fail(GLASMA_ERR_INVALID_ARGUMENT, "field path given without E");
    if ((st = write_efield(d, E, e_path))) return st;
  }
  if (j_path) {
    if (!JpStat || !Jp || !JmStat || !Jm) return io_fail(GLASMA_ERR_INVALID_ARGUMENT, "currents path given without currents");
    if ((st = write_currents(d, JpStat, Jp, JmStat, Jm, j_path))) return st;
  }
  return GLASMA_OK;
}

int glasma_read_text_host(int nx, int ny, int nz, double* U, double* E, double* JpStat, double* Jp, double* JmStat,
                          double* Jm, const char* u_path, const char* e_path, const char* j_path) {
  if (!dims_ok(nx, ny, nz)) return io_fail(GLASMA_ERR_BAD_SHAPE, "bad lattice shape");
  const Dims d{nx, ny, nz};
  int st = GLASMA_OK;
  if (u_path) {
    if (!U) return io_fail(GLASMA_ERR_INVALID_ARGUMENT, "links path given without a links buffer");
    if ((st = read_links(d, U, u_path))) return st;
  }
  if (e_path) {
    if (!E) return io_fail(GLASMA_ERR_INVALID_ARGUMENT, "field path given without an E buffer");
    if ((st = read_efield(d, E, e_path))) return st;
  }
  if (j_path) {
    if (!JpStat || !Jp || !JmStat || !Jm) return io_fail(GLASMA_ERR_INVALID_ARGUMENT, "currents path given without buffers");
    if ((st = read_currents(d, JpStat, Jp, JmStat, Jm, j_path))) return st;
  }
  return GLASMA_OK;
}

int glasma_save_text(glasma_lattice* h, const char* u_path, const char* e_path, const char* j_path) {
  if (!h) return io_fail(GLASMA_ERR_INVALID_ARGUMENT, "null lattice handle");
  const Dims d{h->g.nx, h->g.ny, h->g.nz};
  const size_t S = (size_t)d.sites();
  std::vector<double> U, E, JpS, Jp, JmS, Jm;
  int st;
  if (u_path) {
    U.resize(18 * 3 * S);
    if ((st = glasma_download(h, GLASMA_FIELD_U, U.data()))) return io_fail(st, glasma_last_error());
  }
  if (e_path) {
    E.resize(24 * S);
    if ((st = glasma_download(h, GLASMA_FIELD_E, E.data()))) return io_fail(st, glasma_last_error());
  }
  if (j_path) {
    JpS.resize(8 * S);
    Jp.resize(8 * S);
    JmS.resize(8 * S);
    Jm.resize(8 * S);
    if ((st = glasma_download(h, GLASMA_FIELD_JPSTAT, JpS.data())) || (st = glasma_download(h, GLASMA_FIELD_JP, Jp.data())) ||
        (st = glasma_download(h, GLASMA_FIELD_JMSTAT, JmS.data())) || (st = glasma_download(h, GLASMA_FIELD_JM, Jm.data())))
      return io_fail(st, glasma_last_error());
  }
  return glasma_write_text_host(d.nx, d.ny, d.nz, U.data(), E.data(), JpS.data(), Jp.data(), JmS.data(), Jm.data(),
                                u_path, e_path, j_path);
}

int glasma_load_text(glasma_lattice* h, const char* u_path, const char* e_path, const char* j_path) {
  if (!h) return io_fail(GLASMA_ERR_INVALID_ARGUMENT, "null lattice handle");
  const Dims d{h->g.nx, h->g.ny, h->g.nz};
  const size_t S = (size_t)d.sites();
  std::vector<double> U(u_path ? 18 * 3 * S : 0), E(e_path ? 24 * S : 0);
  std::vector<double> JpS(j_path ? 8 * S : 0), Jp(j_path ? 8 * S : 0), JmS(j_path ? 8 * S : 0), Jm(j_path ? 8 * S : 0);
  int st = glasma_read_text_host(d.nx, d.ny, d.nz, U.data(), E.data(), JpS.data(), Jp.data(), JmS.data(), Jm.data(),
                                 u_path, e_path, j_path);
  if (st) return st;  // nothing uploaded unless every file read cleanly
  if (u_path && (st = glasma_upload(h, GLASMA_FIELD_U, U.data()))) return io_fail(st, glasma_last_error());
  if (e_path && (st = glasma_upload(h, GLASMA_FIELD_E, E.data()))) return io_fail(st, glasma_last_error());
  if (j_path && ((st = glasma_upload(h, GLASMA_FIELD_JPSTAT, JpS.data())) || (st = glasma_upload(h, GLASMA_FIELD_JP, Jp.data())) ||
                 (st = glasma_upload(h, GLASMA_FIELD_JMSTAT, JmS.data())) || (st = glasma_upload(h, GLASMA_FIELD_JM, Jm.data()))))
    return io_fail(st, glasma_last_error());
  return glasma_synchronize(h) ? io_fail(GLASMA_ERR_CUDA, glasma_last_error()) : GLASMA_OK;
}

int glasma_save_binary(glasma_lattice* h, const char* path) {
  if (!h || !path) return io_fail(GLASMA_ERR_INVALID_ARGUMENT, "null argument");
  BinHeader hd;
  std::memset(&hd, 0, sizeof(hd));
  std::memcpy(hd.magic, kMagic, 8);
  hd.version = 1;
  hd.nx = h->g.nx;
  hd.ny = h->g.ny;
  hd.nz = h->g.nz;
  for (int k = 0; k < 3; k++) hd.a[k] = h->g.a[k];
  hd.steps_done = h->steps_done;
  FILE* f = std::fopen(path, "wb");
  if (!f) return io_fail(GLASMA_ERR_INVALID_ARGUMENT, std::string("cannot open ") + path + " for writing");
  bool ok = std::fwrite(&hd, sizeof(hd), 1, f) == 1;
  std::vector<double> buf;
  for (int fld : kBinFields) {
    if (!ok) break;
    const size_t n = (size_t)glasma_field_doubles(h, fld);
    buf.resize(n);
    const int st = glasma_download(h, fld, buf.data());
    if (st) {
      std::fclose(f);
      return io_fail(st, glasma_last_error());
    }
    ok = std::fwrite(buf.data(), sizeof(double), n, f) == n;
  }
  ok = (std::fclose(f) == 0) && ok;
  return ok ? GLASMA_OK : io_fail(GLASMA_ERR_INVALID_ARGUMENT, std::string("write failed: ") + path);
}

int glasma_load_binary(glasma_lattice* h, const char* path) {
  if (!h || !path) return io_fail(GLASMA_ERR_INVALID_ARGUMENT, "null argument");
  FILE* f = std::fopen(path, "rb");
  if (!f) return io_fail(GLASMA_ERR_INVALID_ARGUMENT, std::string("cannot open ") + path);
  BinHeader hd;
  if (std::fread(&hd, sizeof(hd), 1, f) != 1 || std::memcmp(hd.magic, kMagic, 8) != 0 || hd.version != 1) {
    std::fclose(f);
    return io_fail(GLASMA_ERR_INVALID_ARGUMENT, std::string(path) + ": not a binary configuration file");
  }
  if (hd.nx != h->g.nx || hd.ny != h->g.ny || hd.nz != h->g.nz) {
    std::fclose(f);
    return io_fail(GLASMA_ERR_BAD_SHAPE, std::string(path) + ": lattice " + std::to_string(hd.nx) + "x" +
                                             std::to_string(hd.ny) + "x" + std::to_string(hd.nz) +
                                             " does not match the handle's");
  }
  std::vector<std::vector<double>> data(7);
  for (int i = 0; i < 7; i++) {
    const size_t n = (size_t)glasma_field_doubles(h, kBinFields[i]);
    data[i].resize(n);
    if (std::fread(data[i].data(), sizeof(double), n, f) != n) {
      std::fclose(f);
      return io_fail(GLASMA_ERR_INVALID_ARGUMENT, std::string(path) + ": file is truncated");
    }
  }
  std::fclose(f);
  for (int i = 0; i < 7; i++) {
    const int st = glasma_upload(h, kBinFields[i], data[i].data());
    if (st) return io_fail(st, glasma_last_error());
  }
  h->steps_done = hd.steps_done;
  return glasma_synchronize(h) ? io_fail(GLASMA_ERR_CUDA, glasma_last_error()) : GLASMA_OK;
}

}  // extern "C"
