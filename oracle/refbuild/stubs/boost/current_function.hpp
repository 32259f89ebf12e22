// Stand-in for Boost.CurrentFunction (oracle build only).
#pragma once
#define BOOST_CURRENT_FUNCTION __PRETTY_FUNCTION__
