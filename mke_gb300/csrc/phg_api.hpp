// phg_api.hpp -- the guard around every C entry point.  A C++ exception
// (std::bad_alloc from a host array, std::system_error from a thread or a
// mutex) must not unwind into a C caller; inside PHG_API_BEGIN / PHG_API_END
// it becomes PHG_ERR_HOST with its message in phg_last_error().
#pragma once

namespace phg {
// call only from a catch block: records the active exception, returns PHG_ERR_HOST
int api_exception() noexcept;
}  // namespace phg

#define PHG_API_BEGIN try {
#define PHG_API_END        \
    }                      \
    catch (...) {          \
        return phg::api_exception(); \
    }
#define PHG_API_END_VOID   \
    }                      \
    catch (...) {          \
        phg::api_exception(); \
    }
