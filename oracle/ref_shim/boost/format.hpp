/* Minimal stand-in for boost::format: collects the arguments after the
 * format string; only used by the reference for log messages (test oracle only). */
#pragma once
#include <ostream>
#include <sstream>
#include <string>
namespace boost {
class format {
  public:
    explicit format(const char* s) : s_(s) {}
    explicit format(const std::string& s) : s_(s) {}
    template <class T>
    format& operator%(const T& v) {
        std::ostringstream o;
        o << v;
        s_ += " " + o.str();
        return *this;
    }
    std::string str() const { return s_; }
  private:
    std::string s_;
};
inline std::string str(const format& f) { return f.str(); }
inline std::ostream& operator<<(std::ostream& o, const format& f) { return o << f.str(); }
}  // namespace boost
