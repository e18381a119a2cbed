// Stand-in for fmt (test infrastructure for oracle/_ref). The reference only declares formatter
// specialisations and prints diagnostics; formatting here produces nothing.
#pragma once
#include <stdexcept>
#include <string>

namespace fmt {
struct format_parse_context {
    using iterator = const char*;
    const char* b = nullptr;
    constexpr const char* begin() const { return b; }
    constexpr const char* end() const { return b; }
};
struct format_context {
    struct iterator {
        iterator& operator*() { return *this; }
        iterator& operator++() { return *this; }
        iterator operator++(int) { return *this; }
        template <typename T> iterator& operator=(const T&) { return *this; }
    };
    iterator out() { return {}; }
};
struct format_error : std::runtime_error {
    using std::runtime_error::runtime_error;
};
template <typename T, typename Char = char, typename Enable = void>
struct formatter {
    constexpr const char* parse(format_parse_context& ctx) { return ctx.begin(); }
    template <typename Ctx>
    auto format(const T&, Ctx& ctx) const { return ctx.out(); }
};
template <typename Out, typename... A>
inline Out format_to(Out out, A&&...) { return out; }
template <typename... A>
inline std::string format(A&&...) { return {}; }
template <typename... A>
inline void println(A&&...) {}
template <typename... A>
inline void print(A&&...) {}
}
