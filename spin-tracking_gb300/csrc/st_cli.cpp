// spintrack CLI: the drop-in for the reference's `./main params.txt out.bin`
// (main.cpp:19-43): parse the params file, run mainAnalysis on the GPU and
// write output format 'A'.
//
//   spintrack PARAMS OUT [--kernel plain|persistent] [--device N]
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "spintrack.h"

int main(int argc, char** argv) {
  if (argc < 3) {
    std::printf("invalid input options\nExpects ./spintrack parameterFile outputFile "
                "[--kernel plain|persistent] [--device N]\n");
    return 2;
  }
  int kernel = ST_KERNEL_PERSISTENT;
  int device = 0;
  for (int i = 3; i < argc; ++i) {
    if (!std::strcmp(argv[i], "--kernel") && i + 1 < argc) {
      const char* k = argv[++i];
      kernel = !std::strcmp(k, "plain") ? ST_KERNEL_PLAIN : ST_KERNEL_PERSISTENT;
    } else if (!std::strcmp(argv[i], "--device") && i + 1 < argc) {
      device = std::atoi(argv[++i]);
    }
  }
  st_options opt;
  int rc = st_parse_params(argv[1], &opt);
  if (rc == ST_ERR_IO) std::fprintf(stderr, "warning: %s\n", st_last_error());
  else if (rc != ST_OK) {
    std::fprintf(stderr, "error: %s\n", st_last_error());
    return 1;
  }
  const auto t0 = std::chrono::steady_clock::now();
  double run_s = 0.0;
  rc = st_main_analysis(&opt, argv[2], device, kernel, &run_s);
  const auto t1 = std::chrono::steady_clock::now();
  if (rc != ST_OK) {
    std::fprintf(stderr, "error %d: %s\n", rc, st_last_error());
    return 1;
  }
  std::printf("windows: %.3f s\n", run_s);
  std::printf("%lld\n", (long long)std::chrono::duration_cast<std::chrono::milliseconds>(t1 - t0).count());
  return 0;
}
