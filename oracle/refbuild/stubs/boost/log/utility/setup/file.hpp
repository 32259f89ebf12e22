#pragma once
#include <boost/log/core.hpp>
