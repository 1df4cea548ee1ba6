/*
 * The euler app's controls file: brace blocks of `key value...` lines with
 * `#` comments (the reader of src/util/util.cpp:18-79; keys of
 * src/field/field.cpp:25-80 Controls::enroll, src/solvers/properties.cpp
 * Fluid::enroll, apps/euler/euler.cpp:35-50).  Blocks other than the ones
 * asked for are skipped, as the reference skips blocks no solver enrolled.
 */
#ifndef NSEM_DRIVER_CONTROLS_H
#define NSEM_DRIVER_CONTROLS_H

#include <map>
#include <string>
#include <vector>

namespace nsem_driver {

class Controls {
public:
    /* parse `path`; throws std::runtime_error with the file and line */
    explicit Controls(const std::string& path);

    bool has(const std::string& block, const std::string& key) const;
    /* the values of block.key; throws if absent */
    const std::vector<std::string>& values(const std::string& block, const std::string& key) const;
    std::string str(const std::string& block, const std::string& key, const std::string& def) const;
    double num(const std::string& block, const std::string& key, double def) const;
    long integer(const std::string& block, const std::string& key, long def) const;
    /* YES / NO (case-insensitive), as the reference's BoolOption */
    bool flag(const std::string& block, const std::string& key, bool def) const;
    std::vector<double> vec(const std::string& block, const std::string& key, size_t n,
                            const std::vector<double>& def) const;
    const std::string& path() const { return path_; }

private:
    std::string path_;
    std::map<std::string, std::map<std::string, std::vector<std::string>>> blocks_;
};

}  // namespace nsem_driver

#endif
