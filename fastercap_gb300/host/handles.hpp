// Opaque handle types behind the C ABI (shared by api.cpp and server.cpp).
#ifndef FCG_HANDLES_HPP
#define FCG_HANDLES_HPP

#include "../csrc/fcg_internal.hpp"
#include "../../include/fastercap_gb300.h"

struct fcg_context {
    fcg::DeviceContext *dev;
};

struct fcg_problem {
    fcg::DeviceProblem *p;
};

namespace fcg {
// fcg_model_build_on for a server job: the link sources stay in device
// memory (the model's arrays then point there); host/api.cpp
int model_build_device_links(DeviceContext *dev, const char *path, const fcg_build_options *opt, fcg_model **out, char *err,
                             size_t err_len);
}  // namespace fcg

#endif
