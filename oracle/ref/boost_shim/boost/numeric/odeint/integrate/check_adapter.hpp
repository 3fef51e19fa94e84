// Forwarding header of the project's Boost stand-in (test infrastructure).
#include <va_boost_shim.hpp>
