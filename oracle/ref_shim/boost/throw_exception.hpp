/* Stand-in (TEST INFRASTRUCTURE ONLY): the reference includes this header but
 * calls nothing from it. */
#pragma once
