// Command-line options with the semantics of the reference's option parser
// (the vendored tanakh cmdline with J-PET's hooks: lib/cmdline/cmdline.h,
// src/util/cmdline_hooks.cpp, src/util/cmdline_types.h): long options
// `--name=value` / `--name value`, grouped short flags (`-vv` counts twice, the
// last letter of a group may take the next argument), positional arguments,
// `.cfg` files holding one `--name=value` per line ('#' starts a comment),
// options that a config file may not set, and the save rules used when a tool
// writes its options back to a `.cfg`.
#pragma once

#include <cstdint>
#include <map>
#include <memory>
#include <ostream>
#include <stdexcept>
#include <string>
#include <vector>

namespace jpet {
namespace cmd {

enum Flags : unsigned {
  kOptional = 0,
  kRequired = 1,
  kDontSave = 2,
  kAlwaysSave = 4,
};

enum class Kind { Flag, Int, Size, Double, Path, Doubles };

struct Option {
  std::string name;
  char short_name = 0;
  std::string desc;
  Kind kind = Kind::Flag;
  unsigned flags = kOptional;
  bool not_from_file = false;  // ignored when read from a config file
  bool loads_config = false;   // value names a config file to read (-c/--config)
  std::string def;             // default, textual
  std::string value;           // current, textual
  bool has = false;
  int count = 0;
};

// Parse error carrying the messages and the usage text, like cmdline::exception.
struct Error : std::runtime_error {
  explicit Error(const std::string& m) : std::runtime_error(m) {}
};

// Path helpers of cmdline::path (src/util/cmdline_types.h:12-86).
std::string path_wo_ext(const std::string& p);
std::string path_ext(const std::string& p);
std::string path_wo_path(const std::string& p);
std::string path_add_index(const std::string& p, int index, int max_or_digits);

class Parser {
 public:
  void add_flag(const std::string& name, char s, const std::string& desc,
                unsigned flags = kOptional | kDontSave);
  void add(const std::string& name, char s, const std::string& desc, Kind kind, unsigned flags,
           const std::string& def, bool not_from_file = false, bool loads_config = false);
  void footer(const std::string& f) { footer_ = f; }

  // Parses argv; returns false and fills errors() on failure.
  bool parse(int argc, const char* const argv[]);
  // Reference parse_check: usage + exit(0) for no arguments or --help,
  // message + usage + exit(1) on errors.
  void parse_check(int argc, const char* const argv[]);
  // Reads a config file (one argument per line); options marked not_from_file
  // keep their values.  Throws Error if the file cannot be opened.
  void load(const std::string& path);
  // load_accompanying_config (cmdline_hooks.cpp:110-123): <input>.cfg next to
  // each positional argument, if present.
  void load_accompanying_config(bool only_one = false);

  bool exist(const std::string& name) const;
  int count(const std::string& name) const;
  int get_int(const std::string& name) const;
  uint64_t get_size(const std::string& name) const;
  double get_double(const std::string& name) const;
  std::string get_path(const std::string& name) const;
  std::vector<double> get_doubles(const std::string& name) const;
  void set(const std::string& name, const std::string& value);

  const std::vector<std::string>& rest() const { return rest_; }
  const std::vector<std::string>& errors() const { return errors_; }
  std::string usage() const;
  // Writes the options to be saved, one `--name=value` per line (cmdline's
  // parser stream output, used for the phantom tool's .cfg).
  void save(std::ostream& out) const;

 private:
  bool parse_args(const std::vector<std::string>& args, bool from_file);
  void set_option(const std::string& name, const std::string* value, bool from_file);
  Option* find(const std::string& name);
  const Option& get(const std::string& name) const;

  std::map<std::string, std::unique_ptr<Option>> options_;
  std::vector<Option*> ordered_;
  std::vector<std::string> rest_, errors_;
  std::vector<std::string> dir_stack_;
  std::string prog_, footer_;
};

}  // namespace cmd
}  // namespace jpet
