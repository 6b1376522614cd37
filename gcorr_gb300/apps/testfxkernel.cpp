// testfxkernel: one sub-integration from a .conf file and raw antenna files,
// on the GB300 engine.  Same invocation, console output and result files as the
// reference harness (fxkernel/src/testfxkernel.cpp:21-124): reads the config,
// reads one sub-integration per antenna, times process(), writes vis.out and
// runtime.fxkernel.log in the working directory.  Written against the
// reference's class and helper signatures (fxkernel_gxc.h, gxc_common.h).
#include <chrono>
#include <ctime>

#include "fxkernel_gxc.h"
#include "gxc_common.h"

int main(int argc, char *argv[]) {
  if (argc != 2) {
    cout << "Usage:  testfxkernel <config>\n" << endl;
    return 1;
  }
  int nbit, npol, nchan, nant, nfft, subintbytes;
  bool iscomplex;
  double lo, bw;
  vector<string> names, files;
  double **delays = nullptr, *fso = nullptr;
  parseConfig(argv[1], nbit, npol, iscomplex, nchan, nant, lo, bw, nfft, names, files, &delays, &fso);
  cout << "Got COMPLEX " << iscomplex << endl;
  cout << "Got NBIT " << nbit << endl;
  cout << "Got NPOL " << npol << endl;
  cout << "Got NCHAN " << nchan << endl;
  cout << "Got LO " << lo << endl;
  cout << "Got BANDWIDTH " << bw << endl;
  cout << "Got NUMFFTS " << nfft << endl;
  cout << "Got NANT " << nant << endl;
  for (int a = 0; a < nant; a++) cout << "  " << names[a] << ":" << files[a] << endl;

  uint8_t **input = nullptr;
  allocDataHost(&input, nant, nchan, nfft, nbit, npol, iscomplex, subintbytes);
  vector<std::ifstream *> streams;
  for (int a = 0; a < nant; a++) {
    streams.push_back(new std::ifstream(files[a].c_str(), std::ios::binary));
    if (!streams.back()->good()) cerr << "Problem with file " << files[a] << " - does it exist?" << endl;
  }

  FxKernel fx = FxKernel(nant, nchan, nfft, nbit, lo, bw, iscomplex);
  fx.setInputData(input);
  if (readdata(subintbytes, streams, input)) return 1;
  fx.setDelays(delays, fso);

  const auto t0 = std::chrono::high_resolution_clock::now();
  std::time_t now = std::chrono::system_clock::to_time_t(std::chrono::system_clock::now());
  string start = std::ctime(&now);
  start.pop_back();
  fx.process();
  const auto ms = std::chrono::duration_cast<std::chrono::milliseconds>(std::chrono::high_resolution_clock::now() - t0);
  cout << "Run time was " << ms.count() << " milliseconds" << endl;
  fx.saveVisibilities("vis.out");
  std::ofstream log("runtime.fxkernel.log");
  log << "Run time was " << ms.count() << " milliseconds" << endl;
  log << "Start time was " << start << endl;

  for (auto *s : streams) delete s;
  freeDataHost(input, nant);
  for (int a = 0; a < nant; a++) delete[] delays[a];
  delete[] delays;
  delete[] fso;
  return 0;
}
