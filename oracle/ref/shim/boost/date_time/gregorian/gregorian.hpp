// Stand-in for <boost/date_time/gregorian/gregorian.hpp>, used only to compile
// the reference's src/core/configuration.cpp (it prints a module's credit date)
// and src/core/deadline.cpp for the oracle build. Boost is not installed here.
// Only the calls those files make exist; dates are printed as YYYY-Mon-DD.
#ifndef ORACLE_SHIM_BOOST_GREGORIAN_HPP
#define ORACLE_SHIM_BOOST_GREGORIAN_HPP
#include <ctime>
#include <string>
#include <cstdio>
namespace boost {
namespace gregorian {
class days_span {
public:
    explicit days_span(long d) : m_days(d) {}
    long days() const { return m_days; }
private:
    long m_days;
};
class date {
public:
    date(int y, int m, int d) : m_y(y), m_m(m), m_d(d) {}
    int year() const { return m_y; }
    int month() const { return m_m; }
    int day() const { return m_d; }
    long serial() const {
        std::tm t{};
        t.tm_year = m_y - 1900; t.tm_mon = m_m - 1; t.tm_mday = m_d; t.tm_hour = 12;
        return (long)(timegm(&t) / 86400);
    }
    days_span operator-(const date &o) const { return days_span(serial() - o.serial()); }
private:
    int m_y, m_m, m_d;
};
inline std::string to_simple_string(const date &d) {
    static const char *names[] = {"Jan", "Feb", "Mar", "Apr", "May", "Jun",
                                  "Jul", "Aug", "Sep", "Oct", "Nov", "Dec"};
    char buf[32];
    std::snprintf(buf, sizeof(buf), "%04d-%s-%02d", d.year(), names[(d.month() + 11) % 12], d.day());
    return std::string(buf);
}
struct day_clock {
    static date universal_day() {
        std::time_t now = std::time(nullptr);
        std::tm t{};
        gmtime_r(&now, &t);
        return date(t.tm_year + 1900, t.tm_mon + 1, t.tm_mday);
    }
};
class partial_date {
public:
    partial_date(int d, int m) : m_d(d), m_m(m) {}
    date get_date(int y) const { return date(y, m_m, m_d); }
private:
    int m_d, m_m;
};
}  // namespace gregorian
}  // namespace boost
#endif
