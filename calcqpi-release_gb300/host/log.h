// log.h -- log sink of the command-line tools.
//
// Every line is prefixed with "YYYY-MM-DD.HH:MM:SS ", as the reference's AddTimeStamp
// stream buffer does (include/addtimestamp.h); output goes to stdout or, after
// open_append, to the log file (appended).
#pragma once

#include <ctime>
#include <fstream>
#include <iostream>
#include <sstream>
#include <string>

namespace cqpi_cli {

// Line-buffered log sink that prefixes every line with "YYYY-MM-DD.HH:MM:SS ".
class Log {
    std::ostream *os_;
    std::ofstream file_;
    bool bol_ = true;

public:
    Log() : os_(&std::cout) {}
    bool open_append(const std::string &path)
    {
        file_.open(path.c_str(), std::ios::out | std::ios::app);
        if (file_.is_open()) os_ = &file_;
        return file_.is_open();
    }
    Log &operator<<(const std::string &s)
    {
        for (char c : s) {
            if (bol_) {
                char buf[64];
                time_t now = time(nullptr);
                struct tm t;
                localtime_r(&now, &t);
                strftime(buf, sizeof buf, "%Y-%m-%d.%X ", &t);
                *os_ << buf;
            }
            *os_ << c;
            bol_ = (c == '\n');
            if (bol_) os_->flush();
        }
        return *this;
    }
    template <class T>
    Log &operator<<(const T &v)
    {
        std::ostringstream s;
        s << v;
        return *this << s.str();
    }
};

}  // namespace cqpi_cli
