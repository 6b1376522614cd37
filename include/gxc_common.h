/*
 * gxc_common.h — header-only C++ harness helpers with the signatures of the
 * reference's fxkernel/src/common.h:41-60 (parseConfig, allocDataHost,
 * readdata), implemented on the C ABI in gxc.h.  A driver written against the
 * reference (fxkernel/src/testfxkernel.cpp, fxkernel/src/bench_fxkernel.cpp)
 * includes this header and fxkernel_gxc.h instead of common.h and fxkernel.h
 * and links libgxcorr.so.
 *
 * Differences from the reference, all deliberate:
 *  - allocDataHost allocates pinned host memory (the reference does so only in
 *    its CUDA build, common.cpp:22-27) and sizes each buffer with
 *    gxc_input_bytes_per_antenna.  For 2-bit real data that equals the
 *    reference's nchan*2*(nfft+1)*nbit/8*npol (common.cpp:16).  For 8-bit
 *    complex data it is twice that, because each sample carries a real and an
 *    imaginary byte per polarisation.
 *  - parseConfig reports file and line for a malformed line before exiting.
 */
#ifndef GXC_COMMON_H
#define GXC_COMMON_H

#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <iostream>
#include <string>
#include <vector>

#include "gxc.h"

using std::cerr;
using std::cout;
using std::endl;
using std::string;
using std::vector;

/* fxkernel/src/common.h:41-42 */
inline void parseConfig(char *configfilename, int &nbit, int &nPol, bool &iscomplex, int &nchan, int &nant,
                        double &lo, double &bandwidth, int &numffts, vector<string> &antenna,
                        vector<string> &antFiles, double ***delays, double **antfileoffsets) {
  gxc_conffile *cf = nullptr;
  if (gxc_conf_read(configfilename, &cf) != GXC_OK) std::exit(1);
  nbit = gxc_conf_int(cf, "NBIT");
  nPol = gxc_conf_int(cf, "NPOL");
  iscomplex = gxc_conf_int(cf, "COMPLEX") != 0;
  nchan = gxc_conf_int(cf, "NCHAN");
  nant = gxc_conf_int(cf, "NANT");
  numffts = gxc_conf_int(cf, "NUMFFTS");
  lo = gxc_conf_double(cf, "LO");
  bandwidth = gxc_conf_double(cf, "BANDWIDTH");
  std::vector<double> poly((size_t)3 * (nant > 0 ? nant : 0)), fso((size_t)(nant > 0 ? nant : 0));
  gxc_conf_delays(cf, poly.data(), fso.data());
  *delays = new double *[nant > 0 ? nant : 1];
  *antfileoffsets = new double[nant > 0 ? nant : 1];
  for (int a = 0; a < nant; a++) {
    antenna.push_back(gxc_conf_antenna_name(cf, a));
    antFiles.push_back(gxc_conf_antenna_file(cf, a));
    (*delays)[a] = new double[3];
    for (int i = 0; i < 3; i++) (*delays)[a][i] = poly[3 * (size_t)a + i];
    (*antfileoffsets)[a] = fso[a];
  }
  gxc_conf_free(cf);
}

/* fxkernel/src/common.h:55 */
inline void allocDataHost(uint8_t ***data, int numantenna, int numchannels, int numffts, int nbit, int nPol,
                          bool iscomplex, int &subintbytes) {
  gxc_config c;
  gxc_config_init(&c);
  c.nant = numantenna;
  c.nchan = numchannels;
  c.nfft = numffts;
  c.nbit = nbit;
  c.is_complex = iscomplex ? 1 : 0;
  (void)nPol;
  const size_t bytes = gxc_input_bytes_per_antenna(&c);
  subintbytes = (int)bytes;
  cout << "Allocating " << bytes / 1024 / 1024 << " MB per antenna per subint" << endl;
  cout << "          " << bytes * numantenna / 1024 / 1024 << " MB total" << endl;
  *data = new uint8_t *[numantenna];
  for (int a = 0; a < numantenna; a++) {
    void *p = nullptr;
    if (gxc_host_alloc(bytes, &p) != GXC_OK) {
      cerr << "Unable to allocate " << bytes << " bytes. Quitting" << endl;
      std::exit(1);
    }
    (*data)[a] = (uint8_t *)p;
  }
}

/* Frees what allocDataHost allocated. */
inline void freeDataHost(uint8_t **data, int numantenna) {
  for (int a = 0; a < numantenna; a++) gxc_host_free(data[a]);
  delete[] data;
}

/* fxkernel/src/common.h:60: 0 on success, 2 at the end of a file, 1 on a read error. */
inline int readdata(int bytestoread, vector<std::ifstream *> &antStream, uint8_t **inputdata) {
  for (size_t a = 0; a < antStream.size(); a++) {
    std::ifstream &s = *antStream[a];
    s.read((char *)inputdata[a], bytestoread);
    if (!s) {
      if (s.eof()) return 2;
      cerr << "Error: Problem reading data (Read " << s.gcount() << " bytes)" << endl;
      return 1;
    }
  }
  return 0;
}

#endif /* GXC_COMMON_H */
