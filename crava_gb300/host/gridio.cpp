// File formats either side of the inversion (host side).
//
//  * CRAVA FFTGrid binary: FFTGrid::writeCravaFile / readCravaFile
//    (src/fftgrid.cpp:2410-2493): the line "crava_fftgrid_binary", then
//    big-endian binary x0 y0 dx dy (double), nx ny (int32), IL0 XL0 ILStepX
//    ILStepY XLStepX XLStepY angle (double), rnxp nyp nzp (int32) and the
//    rnxp*nyp*nzp floats of the padded real cube.
//  * STORM binary grid (NRLib StormContGrid::WriteToFile / ReadFromFile,
//    libs/nrlib/stormgrid/stormcontgrid.cpp:72-200, volume header
//    libs/nrlib/volume/volume.cpp:381-460): an ASCII header -- format tag,
//    zone, model file name, missing code, variable name, x_min lx y_min ly,
//    four surfaces, lz and the rotation in degrees, ni nj nk -- followed by
//    ni*nj*nk big-endian floats (i fastest) and the barrier count 0.  Only
//    constant surfaces are handled (a surface given as a file name is
//    reported as unsupported).
// The byte order conversions are plain shifts (no host intrinsics).
#include <cctype>
#include <cerrno>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "cravagpu.h"

namespace cg {
void set_error(const char *fmt, ...);
}

namespace {

void put_be32(std::vector<unsigned char> &out, uint32_t v)
{
  for (int s = 24; s >= 0; s -= 8) out.push_back((unsigned char)((v >> s) & 0xffu));
}
void put_be64(std::vector<unsigned char> &out, uint64_t v)
{
  for (int s = 56; s >= 0; s -= 8) out.push_back((unsigned char)((v >> s) & 0xffu));
}
uint32_t get_be32(const unsigned char *p)
{
  return ((uint32_t)p[0] << 24) | ((uint32_t)p[1] << 16) | ((uint32_t)p[2] << 8) | (uint32_t)p[3];
}
uint64_t get_be64(const unsigned char *p)
{
  return ((uint64_t)get_be32(p) << 32) | (uint64_t)get_be32(p + 4);
}
uint32_t f2u(float f) { uint32_t u; std::memcpy(&u, &f, 4); return u; }
float u2f(uint32_t u) { float f; std::memcpy(&f, &u, 4); return f; }
uint64_t d2u(double d) { uint64_t u; std::memcpy(&u, &d, 8); return u; }
double u2d(uint64_t u) { double d; std::memcpy(&d, &u, 8); return d; }

// floats to big-endian bytes and back, in blocks
void floats_to_be(const float *v, size_t n, std::vector<unsigned char> &out)
{
  out.resize(4 * n);
  for (size_t i = 0; i < n; i++) {
    const uint32_t u = f2u(v[i]);
    out[4 * i] = (unsigned char)(u >> 24);
    out[4 * i + 1] = (unsigned char)(u >> 16);
    out[4 * i + 2] = (unsigned char)(u >> 8);
    out[4 * i + 3] = (unsigned char)u;
  }
}
void be_to_floats(const unsigned char *b, size_t n, float *v)
{
  for (size_t i = 0; i < n; i++) v[i] = u2f(get_be32(b + 4 * i));
}

bool write_floats_be(std::ofstream &f, const float *v, size_t n)
{
  const size_t block = 1 << 20;
  std::vector<unsigned char> buf;
  for (size_t o = 0; o < n; o += block) {
    const size_t m = n - o < block ? n - o : block;
    floats_to_be(v + o, m, buf);
    f.write((const char *)buf.data(), (std::streamsize)buf.size());
    if (!f) return false;
  }
  return true;
}
bool read_floats_be(std::ifstream &f, float *v, size_t n)
{
  const size_t block = 1 << 20;
  std::vector<unsigned char> buf(4 * block);
  for (size_t o = 0; o < n; o += block) {
    const size_t m = n - o < block ? n - o : block;
    f.read((char *)buf.data(), (std::streamsize)(4 * m));
    if ((size_t)f.gcount() != 4 * m) return false;
    be_to_floats(buf.data(), m, v + o);
  }
  return true;
}

// std::ostream with precision 14 prints doubles like %.14g
std::string g14(double v)
{
  char s[64];
  std::snprintf(s, sizeof(s), "%.14g", v);
  return s;
}

// whitespace-separated token reader over an ifstream (NRLib ReadNext)
bool next_token(std::ifstream &f, std::string &tok)
{
  tok.clear();
  int c;
  while ((c = f.get()) != EOF && std::isspace(c)) {}
  if (c == EOF) return false;
  tok.push_back((char)c);
  while ((c = f.peek()) != EOF && !std::isspace(c)) tok.push_back((char)f.get());
  return true;
}

bool parse_double(const std::string &t, double &v)
{
  char *end = nullptr;
  errno = 0;
  v = std::strtod(t.c_str(), &end);
  return end && *end == '\0' && errno == 0 && !t.empty();
}

}  // namespace

extern "C" int cg_crava_file_write(const char *path, const float *rvalue, int rnxp, int nyp, int nzp,
                                   const double *geom, const int *nxny)
{
  if (!path || !rvalue || !geom || !nxny || rnxp < 2 || nyp < 1 || nzp < 1) {
    cg::set_error("cg_crava_file_write: bad argument");
    return CG_ERR_ARG;
  }
  std::ofstream f(path, std::ios::out | std::ios::binary | std::ios::trunc);
  if (!f) { cg::set_error("cannot open %s for writing", path); return CG_ERR_ARG; }
  std::vector<unsigned char> h;
  const char *tag = "crava_fftgrid_binary\n";
  h.insert(h.end(), tag, tag + std::strlen(tag));
  for (int t = 0; t < 4; t++) put_be64(h, d2u(geom[t]));          // x0 y0 dx dy
  put_be32(h, (uint32_t)nxny[0]);
  put_be32(h, (uint32_t)nxny[1]);
  for (int t = 4; t < 11; t++) put_be64(h, d2u(geom[t]));         // IL0 XL0 ILStepX ILStepY XLStepX XLStepY angle
  put_be32(h, (uint32_t)rnxp);
  put_be32(h, (uint32_t)nyp);
  put_be32(h, (uint32_t)nzp);
  f.write((const char *)h.data(), (std::streamsize)h.size());
  if (!f || !write_floats_be(f, rvalue, (size_t)rnxp * nyp * nzp)) {
    cg::set_error("write error on %s", path);
    return CG_ERR_STATE;
  }
  return CG_OK;
}

extern "C" int cg_crava_file_read(const char *path, float *rvalue, int rnxp, int nyp, int nzp, double *geom,
                                  int *nxny)
{
  if (!path || !rvalue) { cg::set_error("cg_crava_file_read: bad argument"); return CG_ERR_ARG; }
  std::ifstream f(path, std::ios::in | std::ios::binary);
  if (!f) { cg::set_error("cannot open %s", path); return CG_ERR_ARG; }
  std::string tag;
  std::getline(f, tag);
  if (tag != "crava_fftgrid_binary") { cg::set_error("%s is not a crava_fftgrid_binary file", path); return CG_ERR_ARG; }
  unsigned char b[4 * 8 + 2 * 4 + 7 * 8 + 3 * 4];
  f.read((char *)b, sizeof(b));
  if ((size_t)f.gcount() != sizeof(b)) { cg::set_error("%s: truncated header", path); return CG_ERR_STATE; }
  double g[11];
  int o = 0;
  for (int t = 0; t < 4; t++, o += 8) g[t] = u2d(get_be64(b + o));
  const int nx = (int)get_be32(b + o), ny = (int)get_be32(b + o + 4);
  o += 8;
  for (int t = 4; t < 11; t++, o += 8) g[t] = u2d(get_be64(b + o));
  const int fr = (int)get_be32(b + o), fy = (int)get_be32(b + o + 4), fz = (int)get_be32(b + o + 8);
  if (fr != rnxp || fy != nyp || fz != nzp) {
    cg::set_error("%s holds a %d x %d x %d grid, the model grid is %d x %d x %d (check the padding settings)", path,
                  fr, fy, fz, rnxp, nyp, nzp);
    return CG_ERR_ARG;
  }
  if (!read_floats_be(f, rvalue, (size_t)rnxp * nyp * nzp)) { cg::set_error("%s: truncated data", path); return CG_ERR_STATE; }
  if (geom) std::memcpy(geom, g, sizeof(g));
  if (nxny) { nxny[0] = nx; nxny[1] = ny; }
  return CG_OK;
}

// a surface in the grid header: its file name when it has one, else the constant
static std::string surf_token(const char *file, double z)
{
  const size_t n = strnlen(file, 256);
  return n ? std::string(file, n) : g14(z);
}

extern "C" int cg_storm_write(const char *path, const float *values, int ni, int nj, int nk,
                              const cg_storm_header *hd)
{
  if (!path || !values || !hd || ni < 1 || nj < 1 || nk < 1) { cg::set_error("cg_storm_write: bad argument"); return CG_ERR_ARG; }
  std::ofstream f(path, std::ios::out | std::ios::binary | std::ios::trunc);
  if (!f) { cg::set_error("cannot open %s for writing", path); return CG_ERR_ARG; }
  std::ostringstream s;
  s << "storm_petro_binary\n\n"
    << hd->zone_number << " " << hd->model_file << " " << g14((double)hd->missing_code) << "\n\n"
    << hd->variable << "\n\n"
    << g14(hd->x_min) << " " << g14(hd->lx) << " " << g14(hd->y_min) << " " << g14(hd->ly) << " "
    << surf_token(hd->z_top_file, hd->z_top) << " " << surf_token(hd->z_bot_file, hd->z_bot) << " "
    << surf_token(hd->erosion_top_file, hd->erosion_top) << " " << surf_token(hd->erosion_bot_file, hd->erosion_bot)
    << "\n" << g14(hd->lz) << " " << g14(hd->angle_deg) << "\n"
    << "\n" << ni << " " << nj << " " << nk << "\n";
  const std::string head = s.str();
  f.write(head.data(), (std::streamsize)head.size());
  if (!f || !write_floats_be(f, values, (size_t)ni * nj * nk)) { cg::set_error("write error on %s", path); return CG_ERR_STATE; }
  f << 0;
  return f ? CG_OK : CG_ERR_STATE;
}

// parses the header; leaves the stream at the first data byte
static int storm_header(std::ifstream &f, const char *path, cg_storm_header *hd, int *ni, int *nj, int *nk)
{
  std::string t;
  if (!next_token(f, t)) { cg::set_error("%s: empty file", path); return CG_ERR_ARG; }
  if (t == "storm_petro_ascii") { cg::set_error("%s: STORM ASCII grids are not supported", path); return CG_ERR_UNSUPPORTED; }
  if (t != "storm_petro_binary") { cg::set_error("%s: unknown format %s", path, t.c_str()); return CG_ERR_ARG; }
  cg_storm_header h;
  std::memset(&h, 0, sizeof(h));
  double v;
  if (!next_token(f, t) || !parse_double(t, v)) goto bad;
  h.zone_number = (int)v;
  if (!next_token(f, t)) goto bad;
  std::snprintf(h.model_file, sizeof(h.model_file), "%s", t.c_str());
  if (!next_token(f, t) || !parse_double(t, v)) goto bad;
  h.missing_code = (float)v;
  if (!next_token(f, t)) goto bad;
  std::snprintf(h.variable, sizeof(h.variable), "%s", t.c_str());
  {
    double *dst[10] = {&h.x_min, &h.lx, &h.y_min, &h.ly, &h.z_top, &h.z_bot, &h.erosion_top, &h.erosion_bot, &h.lz,
                       &h.angle_deg};
    char *files[4] = {h.z_top_file, h.z_bot_file, h.erosion_top_file, h.erosion_bot_file};
    for (int q = 0; q < 10; q++) {
      if (!next_token(f, t)) goto bad;
      if (!parse_double(t, *dst[q])) {
        // a surface given as a file (Volume::ReadVolumeFromFile): keep its name
        if (q >= 4 && q < 8 && t.size() < 256) {
          std::snprintf(files[q - 4], 256, "%s", t.c_str());
          *dst[q] = 0.0;
          continue;
        }
        goto bad;
      }
    }
  }
  {
    int dims[3];
    for (int q = 0; q < 3; q++) {
      if (!next_token(f, t) || !parse_double(t, v) || v < 1) goto bad;
      dims[q] = (int)v;
    }
    // DiscardRestOfLine: the binary data start after the end of the dimension line
    int c;
    while ((c = f.get()) != EOF && c != '\n') {}
    if (c == EOF) goto bad;
    *ni = dims[0];
    *nj = dims[1];
    *nk = dims[2];
  }
  if (hd) *hd = h;
  return CG_OK;
bad:
  cg::set_error("%s: malformed STORM header", path);
  return CG_ERR_ARG;
}

extern "C" int cg_storm_read_header(const char *path, cg_storm_header *hd, int *ni, int *nj, int *nk)
{
  if (!path || !ni || !nj || !nk) { cg::set_error("cg_storm_read_header: bad argument"); return CG_ERR_ARG; }
  std::ifstream f(path, std::ios::in | std::ios::binary);
  if (!f) { cg::set_error("cannot open %s", path); return CG_ERR_ARG; }
  return storm_header(f, path, hd, ni, nj, nk);
}

extern "C" int cg_storm_read(const char *path, float *values, long n)
{
  if (!path || !values) { cg::set_error("cg_storm_read: bad argument"); return CG_ERR_ARG; }
  std::ifstream f(path, std::ios::in | std::ios::binary);
  if (!f) { cg::set_error("cannot open %s", path); return CG_ERR_ARG; }
  int ni = 0, nj = 0, nk = 0;
  int rc = storm_header(f, path, nullptr, &ni, &nj, &nk);
  if (rc) return rc;
  if ((long)ni * nj * nk != n) { cg::set_error("%s holds %d x %d x %d values, not %ld", path, ni, nj, nk, n); return CG_ERR_ARG; }
  if (!read_floats_be(f, values, (size_t)n)) { cg::set_error("%s: truncated data", path); return CG_ERR_STATE; }
  std::string t;
  if (next_token(f, t) && t != "0") {
    cg::set_error("%s: %s barriers found; only grids without barriers are supported", path, t.c_str());
    return CG_ERR_UNSUPPORTED;
  }
  return CG_OK;
}

// ---------------------------------------------------------------------------
// STORM binary surfaces
// ---------------------------------------------------------------------------
extern "C" int cg_storm_surface_write(const char *path, const double *z, int ni, int nj, double x_min, double y_min,
                                      double lx, double ly)
{
  if (!path || !z || ni < 2 || nj < 2) { cg::set_error("cg_storm_surface_write: bad argument (ni, nj >= 2)"); return CG_ERR_ARG; }
  std::ofstream f(path, std::ios::out | std::ios::binary | std::ios::trunc);
  if (!f) { cg::set_error("cannot open %s for writing", path); return CG_ERR_ARG; }
  std::ostringstream s;
  s << "STORMGRID_BINARY\n\n"
    << ni << " " << nj << " " << g14(lx / (ni - 1)) << " " << g14(ly / (nj - 1)) << "\n"
    << g14(x_min) << " " << g14(x_min + lx) << " " << g14(y_min) << " " << g14(y_min + ly) << "\n";
  const std::string head = s.str();
  f.write(head.data(), (std::streamsize)head.size());
  const size_t n = (size_t)ni * nj;
  std::vector<unsigned char> buf;
  buf.reserve(8 * n);
  for (size_t i = 0; i < n; i++) put_be64(buf, d2u(z[i]));
  f.write((const char *)buf.data(), (std::streamsize)buf.size());
  if (!f) { cg::set_error("write error on %s", path); return CG_ERR_STATE; }
  return CG_OK;
}

// parses a surface header; leaves the stream at the first data byte
static int surface_header(std::ifstream &f, const char *path, int *ni, int *nj, double *x_min, double *y_min,
                          double *lx, double *ly)
{
  std::string t;
  double v[8];
  if (!next_token(f, t) || t != "STORMGRID_BINARY") { cg::set_error("%s is not a STORM binary surface", path); return CG_ERR_ARG; }
  for (int q = 0; q < 8; q++)
    if (!next_token(f, t) || !parse_double(t, v[q])) { cg::set_error("%s: malformed STORM surface header", path); return CG_ERR_ARG; }
  const int n_i = (int)v[0], n_j = (int)v[1];
  const double dx = v[2], dy = v[3], lxv = v[5] - v[4], lyv = v[7] - v[6];
  if (n_i < 2 || n_j < 2) { cg::set_error("%s: %d x %d nodes", path, n_i, n_j); return CG_ERR_ARG; }
  // NRLib's consistency test (|a - b| <= 1e-4 a)
  if (!(std::fabs(lxv / (n_i - 1) - dx) <= 1e-4 * (lxv / (n_i - 1)))) { cg::set_error("%s: dx != lx/(nx-1)", path); return CG_ERR_ARG; }
  if (!(std::fabs(lyv / (n_j - 1) - dy) <= 1e-4 * (lyv / (n_j - 1)))) { cg::set_error("%s: dy != ly/(ny-1)", path); return CG_ERR_ARG; }
  int c;
  while ((c = f.get()) != EOF && c != '\n') {}
  if (c == EOF) { cg::set_error("%s: truncated", path); return CG_ERR_ARG; }
  *ni = n_i;
  *nj = n_j;
  if (x_min) *x_min = v[4];
  if (y_min) *y_min = v[6];
  if (lx) *lx = lxv;
  if (ly) *ly = lyv;
  return CG_OK;
}

extern "C" int cg_storm_surface_read_header(const char *path, int *ni, int *nj, double *x_min, double *y_min,
                                            double *lx, double *ly)
{
  if (!path || !ni || !nj) { cg::set_error("cg_storm_surface_read_header: bad argument"); return CG_ERR_ARG; }
  std::ifstream f(path, std::ios::in | std::ios::binary);
  if (!f) { cg::set_error("cannot open %s", path); return CG_ERR_ARG; }
  return surface_header(f, path, ni, nj, x_min, y_min, lx, ly);
}

extern "C" int cg_storm_surface_read(const char *path, double *z, long n)
{
  if (!path || !z) { cg::set_error("cg_storm_surface_read: bad argument"); return CG_ERR_ARG; }
  std::ifstream f(path, std::ios::in | std::ios::binary);
  if (!f) { cg::set_error("cannot open %s", path); return CG_ERR_ARG; }
  int ni = 0, nj = 0;
  int rc = surface_header(f, path, &ni, &nj, nullptr, nullptr, nullptr, nullptr);
  if (rc) return rc;
  if ((long)ni * nj != n) { cg::set_error("%s holds %d x %d nodes, not %ld", path, ni, nj, n); return CG_ERR_ARG; }
  std::vector<unsigned char> buf(8 * (size_t)n);
  f.read((char *)buf.data(), (std::streamsize)buf.size());
  if ((size_t)f.gcount() != buf.size()) { cg::set_error("%s: truncated data", path); return CG_ERR_STATE; }
  for (long i = 0; i < n; i++) z[i] = u2d(get_be64(buf.data() + 8 * i));
  // CheckEndOfFile: nothing but whitespace may follow
  std::string t;
  if (next_token(f, t)) { cg::set_error("%s: file too long", path); return CG_ERR_ARG; }
  return CG_OK;
}
