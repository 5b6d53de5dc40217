// cli_common.h -- helpers shared by the drop-in executables.
//
// The executables keep the reference programs' positional command lines and
// output files; options of this project follow as --name=value after them.
#pragma once
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <sys/stat.h>
#include <vector>

#include "muca.h"

namespace cli {

struct Options {
    std::map<std::string, std::string> kv;
    bool has(const char *k) const { return kv.count(k) != 0; }
    long long num(const char *k, long long def) const
    {
        auto it = kv.find(k);
        return it == kv.end() ? def : std::atoll(it->second.c_str());
    }
    double real(const char *k, double def) const
    {
        auto it = kv.find(k);
        return it == kv.end() ? def : std::atof(it->second.c_str());
    }
    std::string str(const char *k, const std::string &def) const
    {
        auto it = kv.find(k);
        return it == kv.end() ? def : it->second;
    }
};

// Splits argv into positional arguments and --name[=value] options.
inline void parse(int argc, char **argv, std::vector<std::string> &pos, Options &opt)
{
    for (int i = 1; i < argc; ++i) {
        const char *a = argv[i];
        if (std::strncmp(a, "--", 2) == 0) {
            const char *eq = std::strchr(a, '=');
            if (eq)
                opt.kv[std::string(a + 2, eq)] = eq + 1;
            else
                opt.kv[a + 2] = "1";
        } else {
            pos.push_back(a);
        }
    }
}

inline void die(const char *what, muca_ctx *c)
{
    std::fprintf(stderr, "error: %s: %s\n", what, muca_last_error(c));
    std::exit(1);
}

// ./fss/L<L> is where the reference programs read and write their files.
inline void ensure_dir(const std::string &d)
{
    std::string cur;
    for (size_t i = 0; i < d.size(); ++i) {
        cur.push_back(d[i]);
        if (d[i] == '/' || i + 1 == d.size()) mkdir(cur.c_str(), 0755);
    }
}

}  // namespace cli
