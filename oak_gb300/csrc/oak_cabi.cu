// OAK's C interface (assimilation.F90:4885-4935): oak_init / oak_assim / oak_done.
// Placeholder until the init-file driver lands: each call records OAKG_ERR_NOTIMPL.
#include <string>

#include "oakg_internal.cuh"

namespace oakg {
int record_failure(int code, const char* msg);
}

extern "C" {
void oak_init(const char* fname) {
  (void)fname;
  oakg::record_failure(OAKG_ERR_NOTIMPL, "oak_init: init-file driver not available in this build");
}
void oak_assim(int ntime, int n, int r, double* Ef, double* Ea) {
  (void)ntime; (void)n; (void)r; (void)Ef; (void)Ea;
  oakg::record_failure(OAKG_ERR_NOTIMPL, "oak_assim: init-file driver not available in this build");
}
void oak_done(void) {}
}
