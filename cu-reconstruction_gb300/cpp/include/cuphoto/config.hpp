// cuphoto::Config (reference: modules/include/config.hpp:10-33) over the
// flat "key: value" YAML files in data/*.yaml (cv::FileStorage's format as
// those files use it: an optional %YAML header, '#' comments, dotted keys,
// numbers and quoted strings).  OpenCV is not required.
#ifndef CUPHOTO_GB300_CONFIG_HPP
#define CUPHOTO_GB300_CONFIG_HPP

#include <map>
#include <sstream>
#include <string>

namespace cuphoto {

class Config {
public:
    bool set_parameter_file(const std::string& filename);
    // Parses text in the same format (used by tests and generated configs).
    void set_parameter_text(const std::string& text);

    template <typename T> T get(const std::string& key, const T& default_value) const {
        auto it = values.find(key);
        if (it == values.end()) return default_value;
        return convert<T>(it->second);
    }
    template <typename T> T get(const std::string& key) const {
        auto it = values.find(key);
        return it == values.end() ? T() : convert<T>(it->second);
    }
    bool has(const std::string& key) const { return values.count(key) != 0; }

private:
    template <typename T> static T convert(const std::string& s) {
        std::istringstream is(s);
        T v{};
        is >> v;
        return v;
    }
    std::map<std::string, std::string> values;
};

template <> inline std::string Config::convert<std::string>(const std::string& s) { return s; }

}  // namespace cuphoto

#endif
