// Stand-in for BOOST_PP_CAT (oracle build only).
#pragma once
#define BOOST_PP_CAT_I(a, b) a##b
#define BOOST_PP_CAT(a, b) BOOST_PP_CAT_I(a, b)
