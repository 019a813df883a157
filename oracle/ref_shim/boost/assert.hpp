#pragma once
// Stand-in for the one macro used by the math headers.
#include <cassert>
#ifndef BOOST_ASSERT
#define BOOST_ASSERT(expr) assert(expr)
#endif
