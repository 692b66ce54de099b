/* Stand-in (TEST INFRASTRUCTURE ONLY): the filter expression of the reference,
 * severity >= level, is defined in trivial.hpp. */
#pragma once

#include "trivial.hpp"
