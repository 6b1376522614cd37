// PSRDADA data streams as engine input (host side).
//
// The reference's ingest (ingest/src/ingest.c:185-330) writes each station's VDIF payloads, headers
// stripped and frames placed in time order, into a PSRDADA ring buffer behind an ASCII header
// built from a template (ingest/src/dada_header_template_atca.txt): "KEY value  # comment" lines
// in the first HDR_SIZE bytes (4096 by default), with UTC_START, MJD_START and PICOSECONDS filled
// in per observation.  A stream saved from such a ring (header, then the data) holds one antenna's
// samples in exactly the engine's input layout: 2-bit A_t | B_t<<2 | A_t+1<<4 | B_t+1<<6, or 8-bit
// complex A.re, A.im, B.re, B.im.  This file parses the header and reads the data of one stream
// per antenna in sub-integration-sized pieces, as gxc_reader does for raw files.  Attaching to a
// live shared-memory ring needs the psrdada library, which this build does not link.
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <strings.h>

#include <fstream>
#include <string>
#include <vector>

#include "gxc.h"

struct gxc_dada_reader {
  std::vector<std::ifstream *> files;
  std::vector<gxc_dada_header> headers;
  size_t bytes = 0;
  int offset_binary = 0;
};

namespace {

constexpr long long kDefaultHeaderSize = 4096;  // psrdada's default header block

// The value token of `key` (case-sensitive, as psrdada writes them), or false.
bool header_value(const char *text, size_t len, const char *key, std::string *val) {
  size_t i = 0;
  const size_t klen = strlen(key);
  while (i < len && text[i] != '\0') {
    size_t e = i;
    while (e < len && text[e] != '\n' && text[e] != '\0') e++;
    // one line [i, e): skip leading blanks, take the first token, compare with key
    size_t a = i;
    while (a < e && (text[a] == ' ' || text[a] == '\t' || text[a] == '\r')) a++;
    size_t b = a;
    while (b < e && text[b] != ' ' && text[b] != '\t' && text[b] != '\r' && text[b] != '#') b++;
    if (b - a == klen && !strncmp(text + a, key, klen)) {
      size_t v = b;
      while (v < e && (text[v] == ' ' || text[v] == '\t')) v++;
      size_t w = v;
      while (w < e && text[w] != ' ' && text[w] != '\t' && text[w] != '\r' && text[w] != '#') w++;
      if (w > v) {
        val->assign(text + v, w - v);
        return true;
      }
      return false;
    }
    i = e + 1;
  }
  return false;
}

long long get_ll(const char *t, size_t n, const char *k, long long dflt) {
  std::string v;
  if (!header_value(t, n, k, &v)) return dflt;
  char *end = nullptr;
  const long long x = strtoll(v.c_str(), &end, 10);
  return (end && *end == '\0') ? x : dflt;
}

double get_d(const char *t, size_t n, const char *k, double dflt) {
  std::string v;
  if (!header_value(t, n, k, &v)) return dflt;
  char *end = nullptr;
  const double x = strtod(v.c_str(), &end);
  return (end && *end == '\0' && isfinite(x)) ? x : dflt;
}

void get_s(const char *t, size_t n, const char *k, char *out, size_t cap) {
  std::string v;
  out[0] = '\0';
  if (header_value(t, n, k, &v) && v != "unset") snprintf(out, cap, "%s", v.c_str());
}

}  // namespace

extern "C" {

gxc_status gxc_dada_header_value(const char *text, size_t len, const char *key, char *value, size_t value_len) {
  if (!text || !key || !value || value_len == 0) return GXC_ERR_INVALID_ARGUMENT;
  std::string v;
  if (!header_value(text, len, key, &v)) return GXC_ERR_INVALID_ARGUMENT;
  if (v.size() + 1 > value_len) return GXC_ERR_INVALID_ARGUMENT;
  memcpy(value, v.c_str(), v.size() + 1);
  return GXC_OK;
}

gxc_status gxc_dada_parse_header(const char *text, size_t len, gxc_dada_header *out) {
  if (!text || !out) return GXC_ERR_INVALID_ARGUMENT;
  memset(out, 0, sizeof(*out));
  out->hdr_size = get_ll(text, len, "HDR_SIZE", kDefaultHeaderSize);
  out->nbit = (int)get_ll(text, len, "NBIT", -1);
  out->npol = (int)get_ll(text, len, "NPOL", -1);
  out->ndim = (int)get_ll(text, len, "NDIM", -1);
  out->nchan = (int)get_ll(text, len, "NCHAN", -1);
  out->bw_mhz = get_d(text, len, "BW", 0.0);
  out->freq_mhz = get_d(text, len, "FREQ", 0.0);
  out->tsamp_us = get_d(text, len, "TSAMP", 0.0);
  out->bytes_per_second = get_ll(text, len, "BYTES_PER_SECOND", -1);
  out->obs_offset = get_ll(text, len, "OBS_OFFSET", -1);
  out->picoseconds = get_ll(text, len, "PICOSECONDS", -1);
  out->mjd_start = get_d(text, len, "MJD_START", 0.0);
  get_s(text, len, "UTC_START", out->utc_start, sizeof(out->utc_start));
  get_s(text, len, "SOURCE", out->source, sizeof(out->source));
  if (out->hdr_size < 64 || out->hdr_size > (1LL << 30)) return GXC_ERR_INVALID_ARGUMENT;
  return GXC_OK;
}

gxc_status gxc_dada_config(const gxc_dada_header *hdr, gxc_config *cfg) {
  if (!hdr || !cfg) return GXC_ERR_INVALID_ARGUMENT;
  if (hdr->nbit < 1 || !(hdr->bw_mhz != 0.0)) return GXC_ERR_INVALID_ARGUMENT;
  if (hdr->npol != 2) return GXC_ERR_UNSUPPORTED;  // the engine correlates dual-pol streams
  cfg->nbit = hdr->nbit;
  cfg->is_complex = hdr->ndim == 2 ? 1 : 0;
  cfg->bw_hz = fabs(hdr->bw_mhz) * 1e6;
  // FREQ is the band centre; the engine's LO is the band edge of channel 0 (real data: band
  // [LO, LO + bw); complex data: the same edge, channels above bw/2 in FFT order)
  cfg->lo_hz = (hdr->freq_mhz - 0.5 * fabs(hdr->bw_mhz)) * 1e6;
  return GXC_OK;
}

gxc_status gxc_dada_open(const char *const *paths, int nant, size_t bytes_per_read, int offset_binary_8bit,
                         gxc_dada_reader **out) {
  if (!paths || nant < 1 || bytes_per_read == 0 || !out) return GXC_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  gxc_dada_reader *r = new gxc_dada_reader();
  r->bytes = bytes_per_read;
  r->offset_binary = offset_binary_8bit;
  for (int a = 0; a < nant; a++) {
    std::ifstream *f = paths[a] ? new std::ifstream(paths[a], std::ios::binary) : nullptr;
    if (!f || !f->good()) {
      fprintf(stderr, "gxc_dada_open: cannot open %s\n", paths[a] ? paths[a] : "(null)");
      delete f;
      gxc_dada_close(r);
      return GXC_ERR_INVALID_ARGUMENT;
    }
    r->files.push_back(f);
    // the header: its first block, then the rest if HDR_SIZE says it is longer
    std::vector<char> text((size_t)kDefaultHeaderSize + 1, '\0');
    f->read(text.data(), kDefaultHeaderSize);
    const size_t got = (size_t)f->gcount();
    gxc_dada_header h;
    if (gxc_dada_parse_header(text.data(), got, &h) != GXC_OK || (long long)got < (h.hdr_size < kDefaultHeaderSize ? h.hdr_size : kDefaultHeaderSize)) {
      fprintf(stderr, "gxc_dada_open: %s: no valid DADA header\n", paths[a]);
      gxc_dada_close(r);
      return GXC_ERR_INVALID_ARGUMENT;
    }
    if (h.hdr_size > kDefaultHeaderSize) {
      text.assign((size_t)h.hdr_size + 1, '\0');
      f->clear();
      f->seekg(0);
      f->read(text.data(), h.hdr_size);
      if (f->gcount() != h.hdr_size || gxc_dada_parse_header(text.data(), (size_t)h.hdr_size, &h) != GXC_OK) {
        fprintf(stderr, "gxc_dada_open: %s: truncated DADA header\n", paths[a]);
        gxc_dada_close(r);
        return GXC_ERR_INVALID_ARGUMENT;
      }
    }
    f->clear();
    f->seekg(h.hdr_size);  // the data start right after the header
    r->headers.push_back(h);
  }
  *out = r;
  return GXC_OK;
}

gxc_status gxc_dada_header_of(const gxc_dada_reader *r, int a, gxc_dada_header *out) {
  if (!r || !out || a < 0 || a >= (int)r->headers.size()) return GXC_ERR_INVALID_ARGUMENT;
  *out = r->headers[(size_t)a];
  return GXC_OK;
}

gxc_status gxc_dada_read(gxc_dada_reader *r, uint8_t *const *bufs) {
  if (!r || !bufs) return GXC_ERR_INVALID_ARGUMENT;
  for (size_t a = 0; a < r->files.size(); a++) {
    if (!bufs[a]) return GXC_ERR_INVALID_ARGUMENT;
    std::ifstream &f = *r->files[a];
    f.read(reinterpret_cast<char *>(bufs[a]), (std::streamsize)r->bytes);
    if ((size_t)f.gcount() != r->bytes) return GXC_END_OF_DATA;
    if (r->offset_binary)
      for (size_t i = 0; i < r->bytes; i++) bufs[a][i] ^= 0x80u;  // offset binary -> two's complement
  }
  return GXC_OK;
}

gxc_status gxc_dada_close(gxc_dada_reader *r) {
  if (!r) return GXC_ERR_INVALID_ARGUMENT;
  for (std::ifstream *f : r->files) delete f;
  delete r;
  return GXC_OK;
}

}  // extern "C"
