// ck_server.cu — continuous-batching serving loop (see ck_server_* in
// include/cudakalman.h).
#include "ck_api_internal.h"

extern "C" {

ck_status ck_server_create(ck_handle*, const ck_options*, const ck_server_config*, ck_server**) {
  return ck::fail(CK_ERR_UNSUPPORTED, "serving loop not built yet");
}
ck_status ck_server_submit(ck_server*, int64_t, const ck_batch_in*) {
  return ck::fail(CK_ERR_UNSUPPORTED, "serving loop not built yet");
}
ck_status ck_server_poll(ck_server*, int64_t*, ck_batch_out*, int32_t, double*, int32_t) {
  return ck::fail(CK_ERR_UNSUPPORTED, "serving loop not built yet");
}
ck_status ck_server_stats(ck_server*, int64_t*, int64_t*, int64_t*, int64_t*) {
  return ck::fail(CK_ERR_UNSUPPORTED, "serving loop not built yet");
}
ck_status ck_server_destroy(ck_server*) { return CK_OK; }

}  // extern "C"
