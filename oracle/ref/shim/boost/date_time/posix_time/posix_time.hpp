// Stand-in for <boost/date_time/posix_time/posix_time.hpp>: the reference's
// src/core/deadline.cpp includes it but calls nothing from it.
#ifndef ORACLE_SHIM_BOOST_POSIX_TIME_HPP
#define ORACLE_SHIM_BOOST_POSIX_TIME_HPP
#endif
