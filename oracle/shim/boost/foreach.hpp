// Minimal stand-in for Boost.Foreach, used only to compile the reference
// sources into the oracle library (oracle/_ref).  Project-written.
#pragma once
#include <cassert>
#define BOOST_FOREACH(VAR, COL) for (VAR : COL)
