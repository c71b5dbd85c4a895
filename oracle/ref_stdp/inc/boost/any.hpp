/* Harness shim (test infrastructure only): Boost is not installed here, and
 * the reference's learning-rule sources use only boost::any and
 * boost::any_cast, which std::any provides with the same meaning. */
#pragma once
#include <any>

namespace boost {
using std::any;
using std::any_cast;
using bad_any_cast = std::bad_any_cast;
} // namespace boost
