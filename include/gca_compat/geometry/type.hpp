// geometry/type.hpp -- include path of the reference header of the same name; the
// definitions are in gca_compat_core.hpp.
#pragma once

#include "../gca_compat_core.hpp"
