// bench_fxkernel: throughput benchmark with the options and report of the
// reference's fxkernel/src/bench_fxkernel.cpp (-nloop, -nbuf, -threads; prints
// "Run time was N milliseconds" and Mbps of packed input), on the GB300 engine.
// Each thread owns one FxKernel (one engine handle) and nbuf copies of the
// random input, and processes nloop*nbuf sub-integrations; all threads share
// the GPU.  Input: 2-bit codes from a seeded Gaussian quantised at +-1 sigma
// (the reference draws N(127, 10) bytes and cuts at 127+-10), or Gaussian
// 8-bit bytes for nbit 8.
#include <getopt.h>

#include <atomic>
#include <chrono>
#include <cstring>
#include <random>
#include <thread>

#include "fxkernel_gxc.h"
#include "gxc_common.h"

static void fill_random(uint8_t *buf, size_t n, int nbit, uint32_t seed) {
  std::mt19937 rng(seed);
  std::normal_distribution<float> g(0.f, 1.f);
  for (size_t i = 0; i < n; i++) {
    if (nbit == 8) {
      const float x = std::round(127.f + 10.f * g(rng));
      buf[i] = (uint8_t)(x < 0.f ? 0.f : (x > 255.f ? 255.f : x));
    } else {
      uint8_t byte = 0;
      for (int j = 0; j < 4; j++) {
        const float x = g(rng);
        const uint8_t code = x >= 1.f ? 3 : (x <= -1.f ? 0 : (x > 0.f ? 2 : 1));
        byte |= (uint8_t)(code << (2 * j));
      }
      buf[i] = byte;
    }
  }
}

int main(int argc, char *argv[]) {
  int nloop = 2, nbuf = 5, nthread = 1;
  static struct option opts[] = {{"nloop", 1, 0, 'n'}, {"nbuf", 1, 0, 'b'}, {"threads", 1, 0, 't'},
                                 {"help", 0, 0, 'h'}, {0, 0, 0, 0}};
  while (true) {
    const int o = getopt_long_only(argc, argv, "n:t:b:h", opts, nullptr);
    if (o == -1) break;
    if (o == 'n') nloop = std::atoi(optarg);
    else if (o == 'b') nbuf = std::atoi(optarg);
    else if (o == 't') nthread = std::atoi(optarg);
    else if (o == 'h') {
      printf("Usage: bench_fxkernel [options] <config>\n");
      printf("  -n/-nloop <n>      Number of loops to process\n");
      printf("  -b/-nbuf <n>       Number of sub-integration buffers to cycle through\n");
      printf("  -t/-threads <t>    Number threads to launch\n");
      return 1;
    }
  }
  if (argc != optind + 1 || nloop < 1 || nbuf < 1 || nthread < 1) {
    cout << "Usage:  bench_fxkernel <config>\n" << endl;
    return 1;
  }
  int nbit, npol, nchan, nant, nfft, subintbytes;
  bool iscomplex;
  double lo, bw;
  vector<string> names, files;
  double **delays = nullptr, *fso = nullptr;
  parseConfig(argv[optind], nbit, npol, iscomplex, nchan, nant, lo, bw, nfft, names, files, &delays, &fso);
  cout << "Got COMPLEX " << iscomplex << endl;
  cout << "Got NBIT " << nbit << endl;
  cout << "Got NPOL " << npol << endl;
  cout << "Got NCHAN " << nchan << endl;
  cout << "Got LO " << lo << endl;
  cout << "Got BANDWIDTH " << bw << endl;
  cout << "Got NUMFFTS " << nfft << endl;
  cout << "Got NANT " << nant << endl;
  const double ts = iscomplex ? 1.0 / bw : 1.0 / (2.0 * bw);
  const int F = iscomplex ? nchan : 2 * nchan;
  const double subint_ms = ts * F * nfft * 1e3;
  cout << "Subint time is " << subint_ms << " msec" << endl;
  cout << "Processing " << subint_ms * nloop * nbuf * nthread / 1000 << " sec " << endl;

  uint8_t **input = nullptr;
  allocDataHost(&input, nant, nchan, nfft, nbit, npol, iscomplex, subintbytes);
  cout << "Initialising data to random values" << endl;
  for (int a = 0; a < nant; a++) fill_random(input[a], (size_t)subintbytes, nbit, 48573u + 7919u * a);

  std::atomic<int> ready(0);
  std::atomic<bool> go(false);
  std::vector<std::thread> th;
  for (int t = 0; t < nthread; t++)
    th.emplace_back([&] {
      std::vector<uint8_t **> data(nbuf);
      for (int j = 0; j < nbuf; j++) {
        allocDataHost(&data[j], nant, nchan, nfft, nbit, npol, iscomplex, subintbytes);
        for (int a = 0; a < nant; a++) std::memcpy(data[j][a], input[a], (size_t)subintbytes);
      }
      FxKernel fx = FxKernel(nant, nchan, nfft, nbit, lo, bw, iscomplex);
      fx.setDelays(delays, fso);
      ready++;
      while (!go.load()) std::this_thread::yield();
      for (int i = 0; i < nloop; i++)
        for (int j = 0; j < nbuf; j++) {
          fx.setInputData(data[j]);
          fx.process();
        }
      for (int j = 0; j < nbuf; j++) freeDataHost(data[j], nant);
    });
  while (ready.load() < nthread) std::this_thread::yield();
  cout << "Go" << endl;
  const auto t0 = std::chrono::high_resolution_clock::now();
  go = true;
  for (auto &t : th) t.join();
  const auto dt = std::chrono::high_resolution_clock::now() - t0;
  const auto ms = std::chrono::duration_cast<std::chrono::milliseconds>(dt);
  const double secs = std::chrono::duration<double>(dt).count();
  cout << "Run time was " << ms.count() << " milliseconds" << endl;
  const double bits = (double)subintbytes * nloop * nbuf * nthread * 8.0 * nant;
  cout << "    " << bits / secs / 1e6 << " Mbps" << endl;
  freeDataHost(input, nant);
  for (int a = 0; a < nant; a++) delete[] delays[a];
  delete[] delays;
  delete[] fso;
  return 0;
}
