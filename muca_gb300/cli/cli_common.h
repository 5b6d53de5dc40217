// cli_common.h -- helpers shared by the drop-in executables.
//
// The executables keep the reference programs' positional command lines and
// output files; options of this project follow as --name=value after them.
#pragma once
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstdint>
#include <cstring>
#include <fstream>
#include <iomanip>
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

// Weight files.  The reference reads them unchecked: a missing file only
// prints "!error!" and the run goes on with zero weights
// (produce2_multigpu.cu:210-213), a short or non-numeric file leaves zeros
// where the read stopped, and the while(!eof) loop writes one entry past the
// array on a trailing newline (:216-220; the continuing file, one value per
// line, :223-235).  Here a file must hold exactly N+1 finite values (for
// the pair format, "i lnW" with i = 0..N in order); anything else is
// reported with the first offending token and the program exits with
// status 3 before it touches the GPU.
inline bool read_tokens(const std::string &path, std::vector<std::string> &tok, std::string &why)
{
    FILE *f = std::fopen(path.c_str(), "r");
    if (!f) {
        why = path + ": cannot open";
        return false;
    }
    char buf[256];
    while (std::fscanf(f, "%255s", buf) == 1) tok.emplace_back(buf);
    std::fclose(f);
    return true;
}

inline bool parse_real(const std::string &t, double &v)
{
    char *end = nullptr;
    v = std::strtod(t.c_str(), &end);
    return end && *end == '\0' && end != t.c_str() && std::isfinite(v);
}

// "i lnW" pairs (produce2_multigpu.cu:214-220)
inline bool read_weight_pairs(const std::string &path, unsigned N, std::vector<double> &w, std::string &why)
{
    std::vector<std::string> tok;
    if (!read_tokens(path, tok, why)) return false;
    w.assign((size_t)N + 1, 0.0);
    for (size_t k = 0; k < tok.size(); k += 2) {
        const size_t i = k / 2;
        char *end = nullptr;
        const long idx = std::strtol(tok[k].c_str(), &end, 10);
        if (!end || *end != '\0' || idx != (long)i) {
            why = path + ": entry " + std::to_string(i) + ": index '" + tok[k] + "' (expected " +
                  std::to_string(i) + ")";
            return false;
        }
        if (i > N) {
            why = path + ": more than N+1 = " + std::to_string(N + 1) + " entries";
            return false;
        }
        if (k + 1 >= tok.size() || !parse_real(tok[k + 1], w[i])) {
            why = path + ": entry " + std::to_string(i) + ": value '" + (k + 1 < tok.size() ? tok[k + 1] : "") +
                  "' is not a finite number";
            return false;
        }
    }
    if (tok.size() != 2 * ((size_t)N + 1)) {
        why = path + ": " + std::to_string(tok.size() / 2) + " entries, expected N+1 = " + std::to_string(N + 1);
        return false;
    }
    return true;
}

// one value per line (the continuing file, muca_delta_multigpu.cu:223-235)
inline bool read_weight_column(const std::string &path, unsigned N, std::vector<double> &w, std::string &why)
{
    std::vector<std::string> tok;
    if (!read_tokens(path, tok, why)) return false;
    if (tok.size() != (size_t)N + 1) {
        why = path + ": " + std::to_string(tok.size()) + " values, expected N+1 = " + std::to_string(N + 1);
        return false;
    }
    w.assign((size_t)N + 1, 0.0);
    for (size_t i = 0; i <= N; ++i)
        if (!parse_real(tok[i], w[i])) {
            why = path + ": value " + std::to_string(i) + " '" + tok[i] + "' is not a finite number";
            return false;
        }
    return true;
}

inline void die_io(const std::string &why)
{
    std::fprintf(stderr, "error: weight file: %s\n", why.c_str());
    std::exit(3);
}

// Chain files (no reference counterpart: the reference saves no lattice,
// and produce_gpu always starts from fresh random spins,
// produce2_multigpu.cu:126-140).  A weight run's final lattices can start a
// production run, so that the chains begin where the converged
// multicanonical walk left them, spread over E_Delta, instead of all near
// E_Delta = 2N/3.  Format: the 8 bytes "MUCACHN1", u32 L, u32 chains (little
// endian), then chains * L * L int8 spins in {-1, 0, +1}, [chain][site],
// site = row * L + col.
inline bool write_chains(const std::string &path, uint32_t L, uint32_t chains, const std::vector<int8_t> &lat,
                         std::string &why)
{
    FILE *f = std::fopen(path.c_str(), "wb");
    if (!f) {
        why = path + ": cannot create";
        return false;
    }
    const uint32_t hdr[2] = {L, chains};
    bool ok = std::fwrite("MUCACHN1", 1, 8, f) == 8 && std::fwrite(hdr, 4, 2, f) == 2 &&
              std::fwrite(lat.data(), 1, lat.size(), f) == lat.size();
    ok = (std::fclose(f) == 0) && ok;
    if (!ok) why = path + ": write failed";
    return ok;
}

inline bool read_chains(const std::string &path, uint32_t L, uint32_t chains, std::vector<int8_t> &lat,
                        std::string &why)
{
    FILE *f = std::fopen(path.c_str(), "rb");
    if (!f) {
        why = path + ": cannot open";
        return false;
    }
    char magic[8];
    uint32_t hdr[2] = {0, 0};
    bool ok = std::fread(magic, 1, 8, f) == 8 && std::memcmp(magic, "MUCACHN1", 8) == 0 && std::fread(hdr, 4, 2, f) == 2;
    if (!ok) {
        std::fclose(f);
        why = path + ": not a chain file";
        return false;
    }
    if (hdr[0] != L || hdr[1] != chains) {
        std::fclose(f);
        why = path + ": holds " + std::to_string(hdr[1]) + " chains of L=" + std::to_string(hdr[0]) + ", expected " +
              std::to_string(chains) + " of L=" + std::to_string(L);
        return false;
    }
    lat.assign((size_t)chains * L * L, 0);
    ok = std::fread(lat.data(), 1, lat.size(), f) == lat.size();
    char extra;
    const bool trailing = std::fread(&extra, 1, 1, f) == 1;
    std::fclose(f);
    if (!ok || trailing) {
        why = path + ": " + (ok ? "trailing bytes" : "truncated");
        return false;
    }
    for (size_t i = 0; i < lat.size(); ++i)
        if (lat[i] < -1 || lat[i] > 1) {
            why = path + ": spin " + std::to_string(i) + " is " + std::to_string((int)lat[i]) + ", not in {-1, 0, 1}";
            return false;
        }
    return true;
}

inline void die_chains(const std::string &why)
{
    std::fprintf(stderr, "error: chain file: %s\n", why.c_str());
    std::exit(3);
}

// ./fss/L<L> is where the reference programs read and write their files.
// The reference's commented-out histogram output (muca_delta_multigpu.cu:
// 528-541): one line per E_Delta bin, "i lnW[i] H[i]", lnW with 10
// significant digits as in the weight files.
inline bool write_hist_dump(const std::string &path, const std::vector<double> &lnw, const std::vector<uint64_t> &h,
                            std::string &why)
{
    if (lnw.size() != h.size()) {
        why = path + ": " + std::to_string(lnw.size()) + " weights for " + std::to_string(h.size()) + " bins";
        return false;
    }
    std::ofstream f(path.c_str());
    if (!f) {
        why = path + ": cannot be opened for writing";
        return false;
    }
    for (size_t i = 0; i < h.size(); ++i)
        f << static_cast<int>(i) << " " << std::setprecision(10) << lnw[i] << " " << h[i] << "\n";
    f.close();
    if (!f) {
        why = path + ": write failed";
        return false;
    }
    return true;
}

inline void ensure_dir(const std::string &d)
{
    std::string cur;
    for (size_t i = 0; i < d.size(); ++i) {
        cur.push_back(d[i]);
        if (d[i] == '/' || i + 1 == d.size()) mkdir(cur.c_str(), 0755);
    }
}

}  // namespace cli
