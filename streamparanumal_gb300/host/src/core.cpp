// settings_t and timers of the GB300 drop-in.
#include <algorithm>
#include <iomanip>
#include <iostream>

#include "core.hpp"

namespace libp {

void settings_t::newSetting(const std::string& shortkey, const std::string& longkey,
                            const std::string& name, const std::string& val,
                            const std::string& description,
                            const std::vector<std::string>& options) {
  LIBP_ABORT("Setting [" << name << "] already exists", settings_.count(name));
  for (auto& kv : settings_)
    LIBP_ABORT("Setting key " << shortkey << "/" << longkey << " already in use",
               kv.second.shortkey == shortkey || kv.second.longkey == longkey);
  settings_[name] = setting_t{shortkey, longkey, name, val, description, options};
  order_.push_back(name);
}

void settings_t::changeSetting(const std::string& name, const std::string& val) {
  auto it = settings_.find(name);
  LIBP_ABORT("Unable to find setting: [" << name << "]", it == settings_.end());
  const auto& opts = it->second.options;
  LIBP_ABORT("Value: " << val << " is not valid for setting " << name,
             !opts.empty() && std::find(opts.begin(), opts.end(), val) == opts.end());
  it->second.val = val;
}

void settings_t::parseSettings(int argc, char** argv) {
  for (int i = 1; i < argc; ++i) {
    const std::string key = argv[i];
    if (key == "-h" || key == "--help") {
      PrintUsage();
      std::exit(LIBP_SUCCESS);
    }
    setting_t* s = nullptr;
    for (auto& kv : settings_)
      if (kv.second.shortkey == key || kv.second.longkey == key) s = &kv.second;
    if (!s) {
      PrintUsage();
      LIBP_FORCE_ABORT("Unrecognized setting: " << key);
    }
    LIBP_ABORT("Setting " << key << " needs a value", i + 1 >= argc);
    changeSetting(s->name, argv[++i]);
  }
}

const std::string& settings_t::raw(const std::string& name) const {
  auto it = settings_.find(name);
  LIBP_ABORT("Unable to find setting: [" << name << "]", it == settings_.end());
  return it->second.val;
}

bool settings_t::compareSetting(const std::string& name, const std::string& token) const {
  return raw(name).find(token) != std::string::npos;
}

void settings_t::reportSetting(const std::string& name) const {
  auto it = settings_.find(name);
  if (it == settings_.end()) return;
  std::cout << std::left << std::setw(30) << name << " : " << it->second.val << "\n";
}

void settings_t::report() const {
  for (auto& n : order_) reportSetting(n);
}

void settings_t::PrintUsage() const {
  std::cout << "Usage:\n\n";
  for (auto& n : order_) {
    const setting_t& s = settings_.at(n);
    std::cout << "[" << s.shortkey << " " << s.longkey << "] " << s.description << " ("
              << s.val << ")";
    if (!s.options.empty()) {
      std::cout << " {";
      for (size_t k = 0; k < s.options.size(); ++k)
        std::cout << (k ? "," : "") << s.options[k];
      std::cout << "}";
    }
    std::cout << "\n";
  }
}

timePoint_t Time() { return std::chrono::steady_clock::now(); }

double ElapsedTime(const timePoint_t start, const timePoint_t end) {
  return std::chrono::duration<double>(end - start).count();
}

}  // namespace libp
