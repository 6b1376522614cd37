// Host-side file formats of the correlator harness: the plain-text .conf
// file, raw packed per-antenna voltage files, the vis.out text dump and
// pinned host buffers.
//
// .conf (fxkernel/src/common.cpp:54-114): one keyword per line, matched
// without regard to case: NBIT, NPOL, COMPLEX, NCHAN, LO (Hz), BANDWIDTH (Hz),
// NUMFFTS, NANT.  The NANT line is followed by NANT antenna lines
// "name file p0 p1 p2 fso": the delay polynomial coefficients of t^2, t and 1
// (seconds, t in FFT intervals) and the file-start offset (seconds); tokens
// after fso are ignored.  Defaults: NPOL 2, COMPLEX 0, NBIT 2.  A line with no
// keyword is an error (the reference exits); an unknown keyword is reported
// on stderr and skipped, as the reference does.
//
// Raw files (fxkernel/src/common.cpp:38-52): each read takes the next
// bytes_per_read bytes of every antenna's file; the end of any file ends the
// stream (the reference's readdata returns 2 there).
//
// vis.out (fxkernel/src/fxkernel.cpp:370-412): one line per channel, the
// channel number (width 5) and the channel-centre frequency
// (c+0.5)/nchan*bw/1e6 MHz (width 11, 6 decimals), then for every baseline
// and product re, im, amplitude, phase (widths 11, 11, 11, 10; 5 decimals).
#include <cuda_runtime.h>
#include <math.h>
#include <stdio.h>
#include <strings.h>

#include <fstream>
#include <iomanip>
#include <sstream>
#include <string>
#include <thread>
#include <vector>

#include "../../include/gxc.h"

struct gxc_conffile {
  int nbit = 2, npol = 2, is_complex = 0, nchan = 0, nant = 0, numffts = 0;
  double lo_hz = 0.0, bw_hz = 0.0;
  std::vector<std::string> names, files;
  std::vector<double> poly, fso;
  std::string err;
};

struct gxc_reader {
  std::vector<std::ifstream *> files;
  size_t bytes = 0;
};

namespace {

template <typename T>
bool read_value(std::istringstream &iss, T &v) {
  return static_cast<bool>(iss >> v);
}

}  // namespace

extern "C" {

gxc_status gxc_conf_read(const char *path, gxc_conffile **out) {
  if (!path || !out) return GXC_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  std::ifstream f(path);
  if (!f.good()) {
    fprintf(stderr, "gxc_conf_read: cannot open %s\n", path);
    return GXC_ERR_INVALID_ARGUMENT;
  }
  gxc_conffile *cf = new gxc_conffile();
  std::string line;
  int pending = 0;
  int lineno = 0;
  auto bad = [&](const std::string &why) {
    fprintf(stderr, "gxc_conf_read: %s:%d: %s\n", path, lineno, why.c_str());
    delete cf;
    return GXC_ERR_INVALID_ARGUMENT;
  };
  while (std::getline(f, line)) {
    lineno++;
    std::istringstream iss(line);
    std::string key;
    if (!(iss >> key)) return bad("could not parse \"" + line + "\"");
    if (pending > 0) {
      std::string file;
      double p[3], fso;
      if (!(iss >> file) || !read_value(iss, p[0]) || !read_value(iss, p[1]) || !read_value(iss, p[2]) ||
          !read_value(iss, fso))
        return bad("antenna line needs: name file p0 p1 p2 fso");
      cf->names.push_back(key);
      cf->files.push_back(file);
      cf->poly.insert(cf->poly.end(), p, p + 3);
      cf->fso.push_back(fso);
      pending--;
      continue;
    }
    const char *k = key.c_str();
    bool ok = true;
    if (!strcasecmp(k, "COMPLEX")) ok = read_value(iss, cf->is_complex);
    else if (!strcasecmp(k, "NBIT")) ok = read_value(iss, cf->nbit);
    else if (!strcasecmp(k, "NPOL")) ok = read_value(iss, cf->npol);
    else if (!strcasecmp(k, "NCHAN")) ok = read_value(iss, cf->nchan);
    else if (!strcasecmp(k, "LO")) ok = read_value(iss, cf->lo_hz);
    else if (!strcasecmp(k, "BANDWIDTH")) ok = read_value(iss, cf->bw_hz);
    else if (!strcasecmp(k, "NUMFFTS")) ok = read_value(iss, cf->numffts);
    else if (!strcasecmp(k, "NANT")) {
      ok = read_value(iss, cf->nant) && cf->nant >= 0;
      if (ok) {
        pending = cf->nant;
        cf->names.clear();
        cf->files.clear();
        cf->poly.clear();
        cf->fso.clear();
      }
    } else {
      fprintf(stderr, "gxc_conf_read: %s:%d: unknown keyword \"%s\"\n", path, lineno, k);
    }
    if (!ok) return bad("bad value for " + key);
  }
  if (pending > 0) return bad("missing antenna lines");
  *out = cf;
  return GXC_OK;
}

gxc_status gxc_conf_config(const gxc_conffile *cf, gxc_config *cfg) {
  if (!cf || !cfg) return GXC_ERR_INVALID_ARGUMENT;
  if (cf->npol != 2) return GXC_ERR_UNSUPPORTED;  // the engine, like fxkernel, takes dual-pol data
  cfg->nant = cf->nant;
  cfg->nchan = cf->nchan;
  cfg->nfft = cf->numffts;
  cfg->nbit = cf->nbit;
  cfg->is_complex = cf->is_complex ? 1 : 0;
  cfg->lo_hz = cf->lo_hz;
  cfg->bw_hz = cf->bw_hz;
  return GXC_OK;
}

int gxc_conf_int(const gxc_conffile *cf, const char *key) {
  if (!cf || !key) return -1;
  if (!strcasecmp(key, "NBIT")) return cf->nbit;
  if (!strcasecmp(key, "NPOL")) return cf->npol;
  if (!strcasecmp(key, "COMPLEX")) return cf->is_complex;
  if (!strcasecmp(key, "NCHAN")) return cf->nchan;
  if (!strcasecmp(key, "NUMFFTS")) return cf->numffts;
  if (!strcasecmp(key, "NANT")) return cf->nant;
  return -1;
}

double gxc_conf_double(const gxc_conffile *cf, const char *key) {
  if (!cf || !key) return NAN;
  if (!strcasecmp(key, "LO")) return cf->lo_hz;
  if (!strcasecmp(key, "BANDWIDTH")) return cf->bw_hz;
  return NAN;
}

const char *gxc_conf_antenna_name(const gxc_conffile *cf, int a) {
  return (cf && a >= 0 && a < (int)cf->names.size()) ? cf->names[a].c_str() : nullptr;
}

const char *gxc_conf_antenna_file(const gxc_conffile *cf, int a) {
  return (cf && a >= 0 && a < (int)cf->files.size()) ? cf->files[a].c_str() : nullptr;
}

gxc_status gxc_conf_delays(const gxc_conffile *cf, double *poly, double *fso) {
  if (!cf) return GXC_ERR_INVALID_ARGUMENT;
  for (size_t i = 0; poly && i < cf->poly.size(); i++) poly[i] = cf->poly[i];
  for (size_t i = 0; fso && i < cf->fso.size(); i++) fso[i] = cf->fso[i];
  return GXC_OK;
}

void gxc_conf_free(gxc_conffile *cf) { delete cf; }

gxc_status gxc_reader_open(const char *const *paths, int nant, size_t bytes_per_read, gxc_reader **out) {
  if (!paths || nant < 1 || !out || !bytes_per_read) return GXC_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  gxc_reader *r = new gxc_reader();
  r->bytes = bytes_per_read;
  for (int a = 0; a < nant; a++) {
    std::ifstream *s = new std::ifstream(paths[a] ? paths[a] : "", std::ios::binary);
    r->files.push_back(s);
    if (!s->good()) {
      fprintf(stderr, "gxc_reader_open: problem with file %s - does it exist?\n", paths[a] ? paths[a] : "(null)");
      gxc_reader_close(r);
      return GXC_ERR_INVALID_ARGUMENT;
    }
  }
  *out = r;
  return GXC_OK;
}

gxc_status gxc_reader_read(gxc_reader *r, uint8_t *const *bufs) {
  if (!r || !bufs) return GXC_ERR_INVALID_ARGUMENT;
  const int n = (int)r->files.size();
  std::vector<int> st(n, 0);
  std::vector<std::thread> th;
  // one reader thread per antenna file: the files are independent streams
  for (int a = 0; a < n; a++)
    th.emplace_back([&, a] {
      std::ifstream *s = r->files[a];
      s->read((char *)bufs[a], (std::streamsize)r->bytes);
      if (!*s) st[a] = s->eof() ? 2 : 1;
    });
  for (auto &t : th) t.join();
  for (int a = 0; a < n; a++)
    if (st[a] == 1) {
      fprintf(stderr, "gxc_reader_read: problem reading antenna %d (read %lld bytes)\n", a,
              (long long)r->files[a]->gcount());
      return GXC_ERR_INVALID_ARGUMENT;
    }
  for (int a = 0; a < n; a++)
    if (st[a] == 2) return GXC_END_OF_DATA;
  return GXC_OK;
}

gxc_status gxc_reader_close(gxc_reader *r) {
  if (!r) return GXC_ERR_INVALID_ARGUMENT;
  for (std::ifstream *s : r->files) delete s;
  delete r;
  return GXC_OK;
}

gxc_status gxc_save_visibilities(const char *path, const float *vis, int nbl, int nchan, double bw_hz) {
  if (!path || (!vis && nbl > 0) || nchan < 1 || nbl < 0) return GXC_ERR_INVALID_ARGUMENT;
  std::ofstream f(path);
  if (!f.good()) return GXC_ERR_INVALID_ARGUMENT;
  for (int c = 0; c < nchan; c++) {
    f << std::setw(5) << c << " " << std::setw(11) << std::fixed << std::setprecision(6)
      << (c + 0.5) / nchan * bw_hz / 1e6;
    f << std::setprecision(5);
    for (int b = 0; b < nbl; b++)
      for (int p = 0; p < 4; p++) {
        const size_t i = (((size_t)b * 4 + p) * nchan + c) * 2;
        const float re = vis[i], im = vis[i + 1];
        f << " " << std::setw(11) << re << " " << std::setw(11) << im;
        f << " " << std::setw(11) << sqrtf(re * re + im * im) << " " << std::setw(10) << atan2f(im, re);
      }
    f << "\n";
  }
  return f.good() ? GXC_OK : GXC_ERR_INVALID_ARGUMENT;
}

gxc_status gxc_host_alloc(size_t bytes, void **out) {
  if (!out) return GXC_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  cudaError_t e = cudaHostAlloc(out, bytes ? bytes : 1, cudaHostAllocDefault);
  if (e != cudaSuccess) {
    fprintf(stderr, "gxc_host_alloc: unable to allocate %zu bytes: %s\n", bytes, cudaGetErrorString(e));
    cudaGetLastError();
    return e == cudaErrorMemoryAllocation ? GXC_ERR_OUT_OF_MEMORY : GXC_ERR_CUDA;
  }
  return GXC_OK;
}

gxc_status gxc_host_free(void *p) {
  if (!p) return GXC_OK;
  return cudaFreeHost(p) == cudaSuccess ? GXC_OK : GXC_ERR_CUDA;
}

}  // extern "C"
