// Option parser with the reference's command-line semantics (see jpet_cmdline.hpp).
#include "jpet_cmdline.hpp"

#include <cctype>
#include <cstdlib>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <sstream>

namespace jpet {
namespace cmd {

namespace {

// integers accept k/m/g suffixes (cmdline_types.h:114-138)
bool parse_long(const std::string& s, long long& out) {
  if (s.empty()) return false;
  char* end = nullptr;
  long long v = std::strtoll(s.c_str(), &end, 10);
  if (end == s.c_str()) return false;
  if (*end) {
    if (end[1]) return false;
    switch (std::tolower(static_cast<unsigned char>(*end))) {
      case 'k': v *= 1000; break;
      case 'm': v *= 1000000; break;
      case 'g': v *= 1000000000; break;
      default: return false;
    }
  }
  out = v;
  return true;
}

bool parse_double(const std::string& s, double& out) {
  if (s.empty()) return false;
  char* end = nullptr;
  double v = std::strtod(s.c_str(), &end);
  if (end == s.c_str() || *end) return false;
  out = v;
  return true;
}

bool valid_value(Kind k, const std::string& v) {
  long long i;
  double d;
  switch (k) {
    case Kind::Int:
    case Kind::Size:
      return parse_long(v, i);
    case Kind::Double:
      return parse_double(v, d);
    case Kind::Doubles: {
      std::istringstream ss(v);
      std::string el;
      while (std::getline(ss, el, ','))
        if (!parse_double(el, d)) return false;
      return true;
    }
    default:
      return true;
  }
}

std::string type_name(Kind k) {
  switch (k) {
    case Kind::Int: return "int";
    case Kind::Size: return "count";
    case Kind::Double: return "float";
    case Kind::Path: return "file";
    case Kind::Doubles: return "float,...";
    default: return "";
  }
}

}  // namespace

std::string path_wo_ext(const std::string& p) {
  auto sep = p.find_last_of("\\/");
  auto dot = p.find_last_of('.');
  if (sep != std::string::npos && dot != std::string::npos && sep > dot) dot = std::string::npos;
  return p.substr(0, dot);
}

std::string path_ext(const std::string& p) {
  auto sep = p.find_last_of("\\/");
  auto dot = p.find_last_of('.');
  if (sep != std::string::npos && dot != std::string::npos && sep > dot) dot = std::string::npos;
  return dot == std::string::npos ? std::string() : p.substr(dot);
}

std::string path_wo_path(const std::string& p) {
  auto sep = p.find_last_of("\\/");
  return p.substr(sep != std::string::npos ? sep + 1 : 0);
}

std::string path_add_index(const std::string& p, int index, int max_or_digits) {
  int n_digits = 1;
  if (max_or_digits > 0) {
    int m = 10;
    while (m <= max_or_digits) {
      ++n_digits;
      m *= 10;
    }
  } else {
    n_digits = max_or_digits;
  }
  std::ostringstream fn;
  fn << p << "_" << std::setw(n_digits) << std::setfill('0') << index;
  return fn.str();
}

void Parser::add_flag(const std::string& name, char s, const std::string& desc, unsigned flags) {
  auto o = std::make_unique<Option>();
  o->name = name;
  o->short_name = s;
  o->desc = desc;
  o->kind = Kind::Flag;
  o->flags = flags;
  ordered_.push_back(o.get());
  options_[name] = std::move(o);
}

void Parser::add(const std::string& name, char s, const std::string& desc, Kind kind,
                 unsigned flags, const std::string& def, bool not_from_file, bool loads_config) {
  auto o = std::make_unique<Option>();
  o->name = name;
  o->short_name = s;
  o->desc = desc;
  o->kind = kind;
  o->flags = flags;
  o->def = def;
  o->value = def;
  o->not_from_file = not_from_file;
  o->loads_config = loads_config;
  ordered_.push_back(o.get());
  options_[name] = std::move(o);
}

Option* Parser::find(const std::string& name) {
  auto it = options_.find(name);
  return it == options_.end() ? nullptr : it->second.get();
}

const Option& Parser::get(const std::string& name) const {
  auto it = options_.find(name);
  if (it == options_.end()) throw Error("there is no flag: --" + name);
  return *it->second;
}

void Parser::set_option(const std::string& name, const std::string* value, bool from_file) {
  Option* o = find(name);
  if (!o) {
    errors_.push_back("undefined option: --" + name);
    return;
  }
  if (o->kind == Kind::Flag) {
    if (value) {
      errors_.push_back("option value is invalid: --" + name + "=" + *value);
      return;
    }
    ++o->count;
    o->has = true;
    return;
  }
  if (!value) {
    errors_.push_back("option needs value: --" + name);
    return;
  }
  if (!valid_value(o->kind, *value)) {
    errors_.push_back("option value is invalid: --" + name + "=" + *value);
    return;
  }
  if (from_file && o->not_from_file) return;  // cmdline::not_from_file hook
  if (o->loads_config) {
    load(*value);
    return;
  }
  o->value = *value;
  o->has = true;
}

bool Parser::parse_args(const std::vector<std::string>& args, bool from_file) {
  std::map<char, std::string> lookup;
  for (auto* o : ordered_)
    if (o->short_name) lookup[o->short_name] = o->name;
  for (size_t i = 0; i < args.size(); ++i) {
    const std::string& a = args[i];
    if (a.compare(0, 2, "--") == 0) {
      auto eq = a.find('=', 2);
      if (eq != std::string::npos) {
        std::string v = a.substr(eq + 1);
        set_option(a.substr(2, eq - 2), &v, from_file);
      } else {
        std::string name = a.substr(2);
        Option* o = find(name);
        if (!o) {
          errors_.push_back("undefined option: --" + name);
          continue;
        }
        if (o->kind != Kind::Flag) {
          if (i + 1 >= args.size()) {
            errors_.push_back("option needs value: --" + name);
            continue;
          }
          set_option(name, &args[++i], from_file);
        } else {
          set_option(name, nullptr, from_file);
        }
      }
    } else if (a.size() > 1 && a[0] == '-') {
      for (size_t j = 1; j + 1 < a.size(); ++j) {
        auto it = lookup.find(a[j]);
        if (it == lookup.end()) {
          errors_.push_back(std::string("undefined short option: -") + a[j]);
          continue;
        }
        set_option(it->second, nullptr, from_file);
      }
      char last = a.back();
      auto it = lookup.find(last);
      if (it == lookup.end()) {
        errors_.push_back(std::string("undefined short option: -") + last);
        continue;
      }
      Option* o = find(it->second);
      if (i + 1 < args.size() && o->kind != Kind::Flag) {
        set_option(it->second, &args[++i], from_file);
      } else {
        set_option(it->second, nullptr, from_file);
      }
    } else if (a.size() == 1 && a[0] == '-') {
      continue;
    } else {
      rest_.push_back(a);
    }
  }
  for (auto* o : ordered_)
    if ((o->flags & kRequired) && !o->has) errors_.push_back("need option: --" + o->name);
  return errors_.empty();
}

bool Parser::parse(int argc, const char* const argv[]) {
  if (!find("help")) add_flag("help", '?', "print this message");
  prog_ = argc > 0 ? argv[0] : "";
  std::vector<std::string> args(argv + 1, argv + argc);
  return parse_args(args, false);
}

void Parser::parse_check(int argc, const char* const argv[]) {
  bool ok = parse(argc, argv);
  if ((argc == 1 && !ok) || exist("help")) {
    std::cerr << usage();
    std::exit(0);
  }
  if (!ok) {
    std::cerr << errors_.front() << std::endl << usage();
    std::exit(1);
  }
}

void Parser::load(const std::string& arg) {
  std::string p = arg;
  if (!dir_stack_.empty() && !p.empty() && p[0] != '/') p = dir_stack_.back() + p;
  std::ifstream in(p);
  if (!in.is_open()) throw Error("cannot open input config file: " + p);
  auto sep = p.find_last_of('/');
  dir_stack_.push_back(sep != std::string::npos ? p.substr(0, sep + 1) : std::string());
  std::vector<std::string> args;
  std::string line;
  while (std::getline(in, line))
    if (!line.empty() && line[0] != '#') args.push_back(line);
  std::vector<std::string> saved_errors;
  saved_errors.swap(errors_);
  std::vector<std::string> saved_rest = rest_;
  parse_args(args, true);
  if (!errors_.empty()) {
    std::cerr << (errors_.size() == 1 ? "warning" : "warnings") << " parsing " << p << ":"
              << std::endl;
    for (auto& e : errors_) std::cerr << "  " << e << std::endl;
  }
  errors_.swap(saved_errors);
  rest_ = saved_rest;
  dir_stack_.pop_back();
}

void Parser::load_accompanying_config(bool only_one) {
  std::vector<std::string> inputs = rest_;
  for (const auto& fn : inputs) {
    std::string cfg = path_wo_ext(fn) + ".cfg";
    std::ifstream in(cfg);
    if (in.is_open()) {
      in.close();
      load(cfg);
      if (only_one) break;
    }
  }
}

bool Parser::exist(const std::string& name) const { return get(name).has; }

int Parser::count(const std::string& name) const {
  const Option& o = get(name);
  return o.kind == Kind::Flag ? o.count : (o.has ? 1 : 0);
}

int Parser::get_int(const std::string& name) const {
  long long v = 0;
  parse_long(get(name).value, v);
  return static_cast<int>(v);
}

uint64_t Parser::get_size(const std::string& name) const {
  long long v = 0;
  parse_long(get(name).value, v);
  return static_cast<uint64_t>(v);
}

double Parser::get_double(const std::string& name) const {
  double v = 0;
  parse_double(get(name).value, v);
  return v;
}

std::string Parser::get_path(const std::string& name) const { return get(name).value; }

std::vector<double> Parser::get_doubles(const std::string& name) const {
  std::vector<double> out;
  std::istringstream ss(get(name).value);
  std::string el;
  while (std::getline(ss, el, ',')) {
    double d;
    if (parse_double(el, d)) out.push_back(d);
  }
  return out;
}

void Parser::set(const std::string& name, const std::string& value) {
  Option* o = find(name);
  if (!o) throw Error("there is no flag: --" + name);
  o->value = value;
}

std::string Parser::usage() const {
  std::ostringstream oss;
  oss << "usage: " << prog_ << " ";
  for (auto* o : ordered_)
    if (o->flags & kRequired) oss << "--" << o->name << "=" << type_name(o->kind) << " ";
  oss << "[options] ... " << footer_ << std::endl << "options:" << std::endl;
  size_t width = 0;
  for (auto* o : ordered_) width = std::max(width, o->name.size());
  for (auto* o : ordered_) {
    if (o->short_name)
      oss << "  -" << o->short_name << ", ";
    else
      oss << "      ";
    oss << "--" << o->name << std::string(width + 4 - o->name.size(), ' ') << o->desc;
    if (o->kind != Kind::Flag) {
      std::string d = o->def;
      if (d.empty() || d == "0" || d == "0.0") d = "auto";
      oss << " (" << type_name(o->kind) << ((o->flags & kRequired) ? "" : " [=" + d + "]")
          << ")";
    }
    oss << std::endl;
  }
  return oss.str();
}

void Parser::save(std::ostream& out) const {
  for (auto* o : ordered_) {
    if (o->flags & kDontSave) continue;
    if (o->kind == Kind::Flag) {
      if (o->count) out << "--" << o->name << std::endl;
    } else if ((o->flags & kAlwaysSave) || o->has || o->value != o->def) {
      out << "--" << o->name << "=" << o->value << std::endl;
    }
  }
}

}  // namespace cmd
}  // namespace jpet
