// Minimal "--key value" / "--key=value" command-line parsing for the drop-in tools (the
// reference uses cxxopts with the same option names and defaults).
#pragma once

#include <cstdlib>
#include <iostream>
#include <map>
#include <string>

class Args {
public:
    Args(int argc, char **argv) {
        for (int i = 1; i < argc; ++i) {
            std::string a = argv[i];
            if (a == "-h" || a == "--help") {
                help_ = true;
                continue;
            }
            if (a.rfind("--", 0) != 0) {
                std::cerr << "unexpected argument: " << a << std::endl;
                std::exit(1);
            }
            a = a.substr(2);
            const auto eq = a.find('=');
            if (eq != std::string::npos) {
                kv_[a.substr(0, eq)] = a.substr(eq + 1);
            } else if (i + 1 < argc) {
                kv_[a] = argv[++i];
            } else {
                std::cerr << "option --" << a << " needs a value" << std::endl;
                std::exit(1);
            }
        }
    }
    bool help() const { return help_; }
    bool has(const std::string &k) const { return kv_.count(k) != 0; }
    std::string str(const std::string &k, const char *def = nullptr) const {
        auto it = kv_.find(k);
        if (it != kv_.end()) return it->second;
        if (def) return def;
        std::cerr << "missing option --" << k << std::endl;
        std::exit(1);
    }
    unsigned long u(const std::string &k, const char *def = nullptr) const {
        return std::strtoul(str(k, def).c_str(), nullptr, 10);
    }
    double d(const std::string &k, const char *def = nullptr) const {
        return std::strtod(str(k, def).c_str(), nullptr);
    }

private:
    bool help_ = false;
    std::map<std::string, std::string> kv_;
};
