/*
 * TEST INFRASTRUCTURE ONLY -- stand-in for boost::core::demangled_name, which the reference's
 * main() uses to name an uncaught exception's type (common/main.cpp:172-173).
 */
#pragma once

#include <cstdlib>
#include <cxxabi.h>
#include <string>
#include <typeinfo>

namespace boost {
namespace core {

inline std::string demangled_name(const std::type_info &t) {
	int status = 0;
	char *s = abi::__cxa_demangle(t.name(), nullptr, nullptr, &status);
	std::string out = status == 0 && s ? s : t.name();
	std::free(s);
	return out;
}

}  // namespace core
}  // namespace boost
