// api_util.h -- error translation at the C ABI: every entry point returns a
// status code and never lets a C++ exception escape.
#pragma once
#include <exception>
#include <new>

#include "../../include/sgdg.h"
#include "sgdg_core.h"

#define API_BEGIN try {
#define API_END                                        \
    return SGDG_OK;                                    \
    }                                                  \
    catch (const sgdg::Error& e) {                     \
        set_error(e.what());                           \
        return e.code;                                 \
    }                                                  \
    catch (const std::bad_alloc&) {                    \
        set_error("host allocation failed");           \
        return SGDG_ENOMEM_BUDGET;                     \
    }                                                  \
    catch (const std::exception& e) {                  \
        set_error(e.what());                           \
        return SGDG_EINVAL;                            \
    }

#define NEED(p)                                                    \
    do {                                                           \
        if (!(p)) throw Error(SGDG_EINVAL, #p " must not be NULL"); \
    } while (0)
