// Opaque handle types behind the C ABI (shared by api.cpp and server.cpp).
#ifndef FCG_HANDLES_HPP
#define FCG_HANDLES_HPP

#include "../csrc/fcg_internal.hpp"

struct fcg_context {
    fcg::DeviceContext *dev;
};

struct fcg_problem {
    fcg::DeviceProblem *p;
};

#endif
