// Test harness (CPU): the driver's Fortran-format file names and the replication of smaller
// files (oak_io.cpp). Usage:
//   io_probe fmt FORMAT K           -> the file name, or ERROR
//   io_probe rep S1 [S2 ...] - T1 [T2 ...]  -> the replicated values of 0, 1, ... (file shape S)
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <string>
#include <vector>

#include "oak_io.h"

int main(int argc, char** argv) {
  if (argc < 2) return 2;
  std::string err;
  if (!strcmp(argv[1], "fmt") && argc == 4) {
    std::string out;
    if (oakg::io::fortran_format(argv[2], atoi(argv[3]), out, err))
      printf("%s\n", out.c_str());
    else
      printf("ERROR %s\n", err.c_str());
    return 0;
  }
  if (!strcmp(argv[1], "rep")) {
    oakg::io::Array a;
    std::vector<int64_t> t;
    int i = 2;
    for (; i < argc && strcmp(argv[i], "-"); i++) a.shape.push_back(atoll(argv[i]));
    for (i++; i < argc; i++) t.push_back(atoll(argv[i]));
    int64_t n = 1;
    for (int64_t s : a.shape) n *= s;
    for (int64_t q = 0; q < n; q++) a.v.push_back((double)q);
    std::vector<double> out;
    if (!oakg::io::replicate(a, t, out, err)) {
      printf("ERROR %s\n", err.c_str());
      return 0;
    }
    for (size_t q = 0; q < out.size(); q++) printf(q ? " %g" : "%g", out[q]);
    printf("\n");
    return 0;
  }
  return 2;
}
