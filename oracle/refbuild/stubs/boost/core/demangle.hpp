#pragma once
#include <string>
namespace boost { namespace core { inline std::string demangle(const char* n) { return n; } } }
