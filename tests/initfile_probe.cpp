// Test harness (CPU): parses an init file with the driver's InitFile and prints every queried
// key as the driver would read it, one line per key.
#include <stdio.h>

#include <string>
#include <vector>

#include "oak_io.h"

int main(int argc, char** argv) {
  if (argc < 2) return 2;
  oakg::io::InitFile f;
  std::string err;
  if (!f.load(argv[1], err)) {
    printf("ERROR %s\n", err.c_str());
    return 0;
  }
  for (int a = 2; a < argc; a++) {
    const std::string key = argv[a];
    std::vector<std::string> items;
    std::vector<double> nums;
    if (!f.has(key)) {
      printf("%s MISSING\n", key.c_str());
    } else if (f.nums(key, nums, err)) {
      printf("%s NUMS", key.c_str());
      for (double x : nums) printf(" %.17g", x);
      printf("\n");
    } else if (f.strs(key, items, err)) {
      printf("%s STRS", key.c_str());
      for (const std::string& s : items) printf(" <%s>", s.c_str());
      printf("\n");
    }
  }
  return 0;
}
