// Stand-in for Boost.Log: every record is discarded (oracle build only).
#pragma once
#include <string>
#include <ostream>
namespace boost { namespace log {
struct null_record {
    template <class T> null_record& operator<<(const T&) { return *this; }
};
namespace sources {
template <class Level> struct severity_logger_mt {};
}
namespace keywords { struct auto_flush_t { bool v; auto_flush_t operator=(bool b) const { return {b}; } };
static const auto_flush_t auto_flush{false}; }
inline void add_file_log(const std::string&, keywords::auto_flush_t) {}
inline void add_file_log(const std::string&) {}
} }
#define BOOST_LOG_SEV(logger, sev) if (true) {} else ::boost::log::null_record()
#define BOOST_LOG_INLINE_GLOBAL_LOGGER_DEFAULT(name, type) \
    struct name { static type& get() { static type l; return l; } };
