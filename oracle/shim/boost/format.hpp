// Minimal printf-style formatter with the boost::format call shape
// (format(fmt) % a % b, .str(), operator<<). Supports %d %u %i %s %f %lf %g
// with optional flags/width/precision and %%. Oracle build only.
#pragma once
#include <cstdio>
#include <ostream>
#include <sstream>
#include <string>
#include <type_traits>

namespace boost {
class format {
public:
    explicit format(const std::string& f) : fmt_(f), pos_(0) { advance(); }
    explicit format(const char* f) : format(std::string(f)) {}

    template <class T>
    format& operator%(const T& v) {
        std::ostringstream os;
        if (pos_ < fmt_.size()) {
            // directive spans [pos_, end_)
            std::string spec = fmt_.substr(pos_, end_ - pos_);
            emit(os, spec, v);
            out_ += os.str();
            pos_ = end_;
            advance();
        } else {
            os << v;
            out_ += os.str();
        }
        return *this;
    }
    std::string str() const { return out_ + rest(); }
    friend std::ostream& operator<<(std::ostream& o, const format& f) { return o << f.str(); }

private:
    std::string fmt_, out_;
    size_t pos_, end_ = 0;

    std::string rest() const {
        std::string r;
        for (size_t i = pos_; i < fmt_.size(); ++i) {
            if (fmt_[i] == '%' && i + 1 < fmt_.size() && fmt_[i + 1] == '%') { r += '%'; ++i; }
            else r += fmt_[i];
        }
        return r;
    }
    // copy literal text up to the next directive; leave pos_ at its '%'
    void advance() {
        while (pos_ < fmt_.size()) {
            if (fmt_[pos_] == '%') {
                if (pos_ + 1 < fmt_.size() && fmt_[pos_ + 1] == '%') { out_ += '%'; pos_ += 2; continue; }
                size_t e = pos_ + 1;
                while (e < fmt_.size() && std::string("diuxXsfFgGeEcp").find(fmt_[e]) == std::string::npos) ++e;
                end_ = (e < fmt_.size()) ? e + 1 : e;
                return;
            }
            out_ += fmt_[pos_++];
        }
    }
    static int precision_of(const std::string& spec) {
        size_t d = spec.find('.');
        if (d == std::string::npos) return -1;
        return std::atoi(spec.c_str() + d + 1);
    }
    template <class T>
    static void emit(std::ostream& os, const std::string& spec, const T& v) {
        int p = precision_of(spec);
        if constexpr (std::is_floating_point<T>::value) {
            os.setf(std::ios::fixed);
            os.precision(p >= 0 ? p : 6);
        }
        os << v;
    }
};
}  // namespace boost
