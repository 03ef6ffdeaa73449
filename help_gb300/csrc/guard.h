// C entry points of the host library must not let a C++ exception reach
// their caller (the exception would cross a C boundary).  The code raises
// only through the standard containers -- std::bad_alloc, std::length_error
// on sizes past what the host can hold -- so every exception is reported as
// the entry point's out-of-memory code.
#ifndef HELP_GUARD_H
#define HELP_GUARD_H

#include <cstdio>

template <class F>
int c_guard(int oom_code, F&& body) {
    try {
        return body();
    } catch (...) {
        return oom_code;
    }
}

// A FILE* that is closed on every way out of the scope.
struct ScopedFile {
    std::FILE* f = nullptr;
    explicit ScopedFile(std::FILE* file) : f(file) {}
    ScopedFile(const ScopedFile&) = delete;
    ScopedFile& operator=(const ScopedFile&) = delete;
    ~ScopedFile() {
        if (f) std::fclose(f);
    }
    int close() {  // fclose's result, once
        const int r = f ? std::fclose(f) : 0;
        f = nullptr;
        return r;
    }
};

#endif
