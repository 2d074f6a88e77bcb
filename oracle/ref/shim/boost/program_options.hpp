// Minimal stand-in for the subset of Boost.Program_options that the FARM
// reference's flag parser uses (options_description, value<T>, variables_map,
// store, parse_command_line, notify). Project-written; it exists only so the
// reference CPU sources compile into the test oracle without Boost installed.
// Only the semantics the reference relies on are provided: "long,s" names,
// valued and flag options, count(), and an exception on unknown options.
#pragma once
#include <map>
#include <memory>
#include <ostream>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

namespace boost {
namespace program_options {

struct value_semantic {
    virtual ~value_semantic() {}
    virtual void assign(const std::string &text) = 0;
};

template <typename T>
struct typed_value : value_semantic {
    T *target;
    explicit typed_value(T *t) : target(t) {}
    void assign(const std::string &text) override {
        std::istringstream is(text);
        T v{};
        is >> v;
        if (is.fail()) throw std::runtime_error("bad value for option");
        *target = v;
    }
};

template <>
inline void typed_value<std::string>::assign(const std::string &text) { *target = text; }

template <typename T>
typed_value<T> *value(T *t) { return new typed_value<T>(t); }

struct option_entry {
    std::string long_name;
    std::string short_name;
    std::shared_ptr<value_semantic> sem;
    std::string help;
};

class options_description;

struct options_init {
    options_description *owner;
    options_init &operator()(const char *name, const char *help);
    options_init &operator()(const char *name, value_semantic *sem, const char *help);
};

class options_description {
public:
    std::vector<option_entry> entries;
    std::string caption;
    explicit options_description(const char *c = "") : caption(c) {}
    options_init add_options() { return options_init{this}; }
    void add(const char *name, value_semantic *sem, const char *help) {
        option_entry e;
        std::string n(name);
        size_t comma = n.find(',');
        if (comma == std::string::npos) {
            e.long_name = n;
        } else {
            e.long_name = n.substr(0, comma);
            e.short_name = n.substr(comma + 1);
        }
        e.sem.reset(sem);
        e.help = help;
        entries.push_back(e);
    }
    const option_entry *find(const std::string &key) const {
        for (auto &e : entries)
            if (e.long_name == key || (!e.short_name.empty() && e.short_name == key)) return &e;
        return nullptr;
    }
};

inline options_init &options_init::operator()(const char *name, const char *help) {
    owner->add(name, nullptr, help);
    return *this;
}
inline options_init &options_init::operator()(const char *name, value_semantic *sem, const char *help) {
    owner->add(name, sem, help);
    return *this;
}

inline std::ostream &operator<<(std::ostream &os, const options_description &d) {
    os << d.caption << ":\n";
    for (auto &e : d.entries) os << "  --" << e.long_name << "  " << e.help << "\n";
    return os;
}

struct parsed_options {
    std::vector<std::pair<const option_entry *, std::string>> items;
};

class variables_map {
public:
    std::map<std::string, std::vector<std::pair<const option_entry *, std::string>>> seen;
    size_t count(const std::string &k) const { return seen.count(k); }
};

inline parsed_options parse_command_line(int argc, char **argv, const options_description &desc) {
    parsed_options out;
    for (int i = 1; i < argc; i++) {
        std::string a(argv[i]);
        std::string key;
        if (a.rfind("--", 0) == 0) key = a.substr(2);
        else if (a.size() >= 2 && a[0] == '-') key = a.substr(1);
        else throw std::runtime_error("positional arguments are not supported");
        std::string inline_val;
        bool has_inline = false;
        size_t eq = key.find('=');
        if (eq != std::string::npos) {
            inline_val = key.substr(eq + 1);
            key = key.substr(0, eq);
            has_inline = true;
        }
        const option_entry *e = desc.find(key);
        if (!e) throw std::runtime_error("unknown option " + a);
        std::string v;
        if (e->sem) {
            if (has_inline) v = inline_val;
            else if (i + 1 < argc) v = argv[++i];
            else throw std::runtime_error("missing value for " + a);
        }
        out.items.push_back({e, v});
    }
    return out;
}

inline void store(const parsed_options &p, variables_map &vm) {
    for (auto &it : p.items) vm.seen[it.first->long_name].push_back(it);
}

inline void notify(variables_map &vm) {
    for (auto &kv : vm.seen)
        for (auto &it : kv.second)
            if (it.first->sem) it.first->sem->assign(it.second);
}

}  // namespace program_options
}  // namespace boost
