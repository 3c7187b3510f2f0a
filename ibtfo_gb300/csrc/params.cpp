// .inp reader compatible with the reference's ParamReader
// (Src/Utils/ParamReader.cpp:14-68, Src/Utils/ParamReader.H:38-59), plus the
// solver-slot keys the reference selects in its Makefiles
// (Test/Sod/Makefile:1-7), which this reader takes from the same file.
//
// Numeric values follow ParamReader::numbers() exactly: lines whose first
// character is '#' are skipped, every space is removed, the key is the text
// before the first '=', and the value is the first match of
// [+-]?(\d*\.\d+|\d+) after it converted with atof (so "1e-5" reads as 1 and
// a key without a number reads as 0).  String values (Scheme = MUSCL) are the
// text after '=' up to a '#', spaces removed.
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <regex>
#include <string>
#include <vector>

#include "../../include/ibtfo.h"

namespace ibtfo {
void set_last_error(const char *msg);
}

struct ibtfo_inp
{
    std::map<std::string, double> numbers;
    std::map<std::string, std::string> strings;
};

namespace {

std::string strip_spaces(std::string s)
{
    s.erase(std::remove(s.begin(), s.end(), ' '), s.end());
    return s;
}

bool parse_lines(const std::vector<std::string> &lines, ibtfo_inp *out)
{
    static const std::regex number("[+-]?(\\d*\\.\\d+|\\d+)");
    for (const std::string &raw : lines)
    {
        if (!raw.empty() && raw[0] == '#')
            continue;
        std::string line = strip_spaces(raw);
        if (!line.empty() && line.back() == '\r')
            line.pop_back();
        const size_t eq = line.find('=');
        const std::string key = line.substr(0, eq);
        const std::string value = (eq == std::string::npos) ? line : line.substr(eq + 1);
        std::smatch m;
        std::string num;
        if (std::regex_search(value, m, number))
            num = m.str();
        out->numbers[key] = atof(num.c_str());
        std::string sv = value.substr(0, value.find('#'));
        out->strings[key] = sv;
    }
    return true;
}

int lookup(const char *name, const char *const *names, int n)
{
    for (int i = 0; i < n; i++)
        if (strcmp(name, names[i]) == 0)
            return i;
    return -1;
}

} // namespace

extern "C" {

ibtfo_status ibtfo_inp_open(const char *path, ibtfo_inp **out)
{
    if (!path || !out)
    {
        ibtfo::set_last_error("ibtfo_inp_open: null argument");
        return IBTFO_EINVAL;
    }
    std::ifstream in(path);
    if (!in)
    {
        ibtfo::set_last_error((std::string("cannot open ") + path).c_str());
        return IBTFO_EINVAL;
    }
    std::vector<std::string> lines;
    std::string s;
    while (std::getline(in, s))
        lines.push_back(s);
    ibtfo_inp *p = new ibtfo_inp();
    parse_lines(lines, p);
    *out = p;
    return IBTFO_OK;
}

ibtfo_status ibtfo_inp_parse(const char *text, ibtfo_inp **out)
{
    if (!text || !out)
    {
        ibtfo::set_last_error("ibtfo_inp_parse: null argument");
        return IBTFO_EINVAL;
    }
    std::vector<std::string> lines;
    const char *b = text;
    while (*b)
    {
        const char *e = strchr(b, '\n');
        if (!e)
        {
            lines.emplace_back(b);
            break;
        }
        lines.emplace_back(b, e - b);
        b = e + 1;
    }
    ibtfo_inp *p = new ibtfo_inp();
    parse_lines(lines, p);
    *out = p;
    return IBTFO_OK;
}

void ibtfo_inp_close(ibtfo_inp *p) { delete p; }

int ibtfo_inp_get(const ibtfo_inp *p, const char *key, double def, double *value)
{
    auto it = p ? p->numbers.find(key) : decltype(p->numbers.end())();
    if (!p || it == p->numbers.end())
    {
        if (value)
            *value = def;
        return 0;
    }
    if (value)
        *value = it->second;
    return 1;
}

int ibtfo_inp_get_string(const ibtfo_inp *p, const char *key, char *buf, int size)
{
    if (!p)
        return 0;
    auto it = p->strings.find(key);
    if (it == p->strings.end())
        return 0;
    if (buf && size > 0)
    {
        strncpy(buf, it->second.c_str(), (size_t)size - 1);
        buf[size - 1] = '\0';
    }
    return 1;
}

ibtfo_status ibtfo_config_from_inp(const ibtfo_inp *p, ibtfo_config *cfg)
{
    if (!p || !cfg)
    {
        ibtfo::set_last_error("ibtfo_config_from_inp: null argument");
        return IBTFO_EINVAL;
    }
    ibtfo_config c = {};
    double v;
    // defaults of the reference drivers, Test/Sod/Sod.cpp:34-48
    ibtfo_inp_get(p, "max_iter", 100000, &v);
    c.max_iter = int(v);
    ibtfo_inp_get(p, "lo_x", 0, &c.lo_x);
    ibtfo_inp_get(p, "lo_y", 0, &c.lo_y);
    ibtfo_inp_get(p, "hi_x", 1, &c.hi_x);
    ibtfo_inp_get(p, "hi_y", 1, &c.hi_y);
    ibtfo_inp_get(p, "N_x", 500, &v);
    c.n_x = int(v);
    ibtfo_inp_get(p, "N_y", 200, &v);
    c.n_y = int(v);
    ibtfo_inp_get(p, "Psy_time", 1.0, &c.psy_time);
    ibtfo_inp_get(p, "CFL_number", 0.3, &c.cfl_number);
    ibtfo_inp_get(p, "num_ghost_cell", 2, &v);
    c.num_ghost_cell = int(v);
    ibtfo_inp_get(p, "gamma", 1.4, &c.gamma);

    static const char *const schemes[] = {"MUSCL", "MHM", "Godunov", "Lax"};
    static const char *const times[] = {"SingleStep", "RK2"};
    static const char *const riemanns[] = {"HLL", "HLLC", "PVRS", "StegerWarming", "HLLC_Toro", "HLL_Toro"};
    static const char *const limiters[] = {"minmod", "VanLeer"};
    static const char *const bounds[] = {"Regular", "IDWBaseGFM", "LinearBaseGFM", "RiemannBaseGFM", "BCGFM", "HBCGFM",
                                         "CCM"};
    static const char *const globals[] = {"Walls", "Periodic"};
    static const char *const precs[] = {"FP64", "FP64_FAST", "FP32_COMPENSATED"};
    struct Slot
    {
        const char *key;
        const char *const *names;
        int n;
        int *dst;
        int def;
    } slots[] = {{"Scheme", schemes, 4, &c.scheme, 0},        {"Riemann", riemanns, 6, &c.riemann, 0},
                 {"Limiter", limiters, 2, &c.limiter, 0},     {"Boundary", bounds, 7, &c.boundary, 0},
                 {"Global_Boundary", globals, 2, &c.global_boundary, 0}, {"Precision", precs, 3, &c.precision, 0},
                 {"Time", times, 2, &c.time_advance, 0}};
    char buf[256];
    for (const Slot &s : slots)
    {
        *s.dst = s.def;
        if (ibtfo_inp_get_string(p, s.key, buf, sizeof buf) && buf[0])
        {
            int k = lookup(buf, s.names, s.n);
            if (k < 0)
            {
                ibtfo::set_last_error((std::string("unknown ") + s.key + " value '" + buf + "'").c_str());
                return IBTFO_EINVAL;
            }
            *s.dst = k;
        }
    }
    *cfg = c;
    return IBTFO_OK;
}

} // extern "C"
