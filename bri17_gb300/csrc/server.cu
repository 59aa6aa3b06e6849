// server.cu -- continuous-batching solve server (placeholder until the
// scheduler lands; every entry point reports BRI17_ERR_INVALID_ARGUMENT).
#include "op.cuh"

extern "C" int bri17_server_create(int64_t, int, bri17_server** s) {
  if (s) *s = nullptr;
  return BRI17_ERR_INVALID_ARGUMENT;
}
extern "C" int bri17_server_destroy(bri17_server*) { return BRI17_OK; }
extern "C" int bri17_server_submit(bri17_server*, const int*, const double*, double, double,
                                   const double*, double*, double, int, int64_t*) {
  return BRI17_ERR_INVALID_ARGUMENT;
}
extern "C" int bri17_server_step(bri17_server*, int*) { return BRI17_ERR_INVALID_ARGUMENT; }
extern "C" int bri17_server_poll(bri17_server*, bri17_request_result*, int, int*) {
  return BRI17_ERR_INVALID_ARGUMENT;
}
extern "C" int bri17_server_cancel(bri17_server*, int64_t) { return BRI17_ERR_INVALID_ARGUMENT; }
extern "C" double bri17_server_clock(const bri17_server*) { return 0.0; }
