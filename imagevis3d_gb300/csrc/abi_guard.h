// The exported functions run their bodies inside GBVR_ABI_TRY ... GBVR_ABI_CATCH
// so that no C++ exception crosses the C boundary: a failed host allocation
// becomes GBVR_ENOMEM and any other exception GBVR_EINVAL, each with its
// message for gbvr_last_error.  Functions returning a size return 0 instead.
#pragma once
#include <exception>
#include <new>
#include <string>

#include "../../include/gbvr.h"

namespace gbvr {
int set_error(int code, const std::string& msg);
}

#define GBVR_ABI_TRY try {
#define GBVR_ABI_CATCH                                                  \
  }                                                                     \
  catch (const std::bad_alloc&) {                                       \
    return gbvr::set_error(GBVR_ENOMEM, "out of host memory");          \
  }                                                                     \
  catch (const std::exception& e) {                                     \
    return gbvr::set_error(GBVR_EINVAL, e.what());                      \
  }
#define GBVR_ABI_CATCH_SIZE          \
  }                                  \
  catch (const std::exception&) {    \
    return 0;                        \
  }
