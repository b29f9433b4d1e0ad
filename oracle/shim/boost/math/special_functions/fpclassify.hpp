// Minimal stand-in for boost::math::isnan.  Project-written.
#pragma once
#include <cmath>
namespace boost { namespace math { using std::isnan; } }
