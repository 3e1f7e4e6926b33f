// cuphoto::Config (reference: config.cpp:8-23) over flat YAML files.
#include "cuphoto/config.hpp"

#include <cstdio>
#include <fstream>

namespace cuphoto {

namespace {

std::string trim(const std::string& s) {
    size_t a = 0, b = s.size();
    while (a < b && (s[a] == ' ' || s[a] == '\t' || s[a] == '\r')) ++a;
    while (b > a && (s[b - 1] == ' ' || s[b - 1] == '\t' || s[b - 1] == '\r')) --b;
    return s.substr(a, b - a);
}

}  // namespace

void Config::set_parameter_text(const std::string& text) {
    std::istringstream in(text);
    std::string line;
    while (std::getline(in, line)) {
        if (!line.empty() && line[0] == '%') continue;  // %YAML:1.0
        bool quoted = false;
        for (size_t i = 0; i < line.size(); ++i) {   // strip comments outside quotes
            if (line[i] == '"') quoted = !quoted;
            if (line[i] == '#' && !quoted) {
                line.resize(i);
                break;
            }
        }
        const size_t colon = line.find(':');
        if (colon == std::string::npos) continue;
        const std::string key = trim(line.substr(0, colon));
        std::string val = trim(line.substr(colon + 1));
        if (key.empty()) continue;
        if (val.size() >= 2 && val.front() == '"' && val.back() == '"') val = val.substr(1, val.size() - 2);
        values[key] = val;
    }
}

bool Config::set_parameter_file(const std::string& filename) {
    std::ifstream f(filename);
    if (!f.is_open()) {
        std::fprintf(stderr, "parameter file %s does not exist.\n", filename.c_str());
        return false;
    }
    std::stringstream ss;
    ss << f.rdbuf();
    set_parameter_text(ss.str());
    return true;
}

}  // namespace cuphoto
