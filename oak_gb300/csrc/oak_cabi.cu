// OAK's C interface (assimilation.F90:4885-4935): oak_init / oak_assim / oak_done.
// oak_init and oak_done manage the library's device context (created on init, released on
// done). The init-file driver behind oak_assim (file I/O, state packing, operator generation)
// is not part of this library; oak_assim records OAKG_ERR_NOTIMPL and points to
// oakg_ens_locanalysis, the numerical core a driver calls.
#include <stdio.h>

#include <mutex>
#include <string>

#include "oakg_internal.cuh"

namespace oakg {
int record_failure(int code, const char* msg);
int context_init_impl();
int release_impl();
void set_ok();
std::mutex& api_mutex();
int& last_status();
}  // namespace oakg

extern "C" {
void oak_init(const char* fname) {
  std::lock_guard<std::mutex> lk(oakg::api_mutex());
  oakg::set_ok();
  FILE* f = fname ? fopen(fname, "r") : nullptr;
  if (!f) {
    std::string msg = std::string("oak_init: cannot read init file '") + (fname ? fname : "(null)") +
                      "'";
    oakg::last_status() = oakg::record_failure(OAKG_ERR_INIT, msg.c_str());
    return;
  }
  fclose(f);
  oakg::last_status() = oakg::context_init_impl();
}

void oak_assim(int ntime, int n, int r, double* Ef, double* Ea) {
  (void)ntime;
  (void)n;
  (void)r;
  (void)Ef;
  (void)Ea;
  std::lock_guard<std::mutex> lk(oakg::api_mutex());
  oakg::set_ok();
  oakg::last_status() = oakg::record_failure(
      OAKG_ERR_NOTIMPL,
      "oak_assim: the init-file driver (observation and model files, operator generation) is "
      "not part of this library; call oakg_ens_locanalysis with the ensemble, the observation "
      "operator and the observations");
}

void oak_done(void) {
  std::lock_guard<std::mutex> lk(oakg::api_mutex());
  oakg::set_ok();
  oakg::last_status() = oakg::release_impl();
}
}
