#pragma once
#include <boost/fusion/container.hpp>
