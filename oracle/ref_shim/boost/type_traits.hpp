// Stand-in for the one boost header the reference's xbar culling headers use
// (boost::is_base_of in dp/rix/core/HandledObject.h); the standard library has it.
#pragma once
#include <type_traits>
namespace boost { using std::is_base_of; }
