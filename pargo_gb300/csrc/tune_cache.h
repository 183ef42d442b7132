// tune_cache.h -- the autotuner's persisted choices (host code only, no CUDA).
//
// The autotuner's choices outlive the context in a JSON file, keyed by
// operation, device and size class, so a fresh context -- an application's
// main, say -- runs the tuned kernel:
//   {"version": 1, "entries": [{"op": "slope_d8", "device": "sm_103 152 NVIDIA GB300",
//     "size_class": 30, "variant": "strip-s6x8-b5", "ms": 2.031}, ...]}
// The file is PARGO_TUNE_CACHE when set (set but empty: no cache), else
// $XDG_CACHE_HOME/pargo_gb300/tune.json, else $HOME/.cache/pargo_gb300/tune.json.
// Entries name variants by their parameters (focal_variant_name); a name
// this build does not know is ignored.

#pragma once

#include <stdio.h>
#include <stdlib.h>
#include <sys/stat.h>
#include <unistd.h>

#include <algorithm>
#include <atomic>
#include <string>
#include <vector>

namespace pargo {

struct TuneEntry {
    std::string op, device, variant;
    int size_class = -1;
    double ms = 0.0;
};

inline std::string tune_cache_path() {
    const char* env = getenv("PARGO_TUNE_CACHE");
    if (env) return std::string(env);
    const char* xdg = getenv("XDG_CACHE_HOME");
    if (xdg && *xdg) return std::string(xdg) + "/pargo_gb300/tune.json";
    const char* home = getenv("HOME");
    if (home && *home) return std::string(home) + "/.cache/pargo_gb300/tune.json";
    return std::string();
}

// A small JSON reader for the cache file: values are objects, arrays,
// strings, numbers, true/false/null; anything malformed ends the read (the
// entries read so far are kept).
struct JsonReader {
    const std::string& t;
    size_t i = 0;
    bool ok = true;
    explicit JsonReader(const std::string& text) : t(text) {}
    void ws() {
        while (i < t.size() && (t[i] == ' ' || t[i] == '\n' || t[i] == '\r' || t[i] == '\t')) i++;
    }
    bool eat(char c) {
        ws();
        if (i < t.size() && t[i] == c) {
            i++;
            return true;
        }
        return false;
    }
    bool str(std::string* out) {
        ws();
        if (i >= t.size() || t[i] != '"') return ok = false;
        i++;
        std::string r;
        while (i < t.size() && t[i] != '"') {
            char c = t[i++];
            if (c == '\\' && i < t.size()) {
                const char e = t[i++];
                if (e == 'n') c = '\n';
                else if (e == 't') c = '\t';
                else if (e == 'u') {  // \uXXXX: kept as '?' (the cache writes none)
                    i = std::min(t.size(), i + 4);
                    c = '?';
                } else c = e;
            }
            r.push_back(c);
        }
        if (i >= t.size()) return ok = false;
        i++;
        if (out) *out = r;
        return true;
    }
    bool num(double* out) {
        ws();
        const char* b = t.c_str() + i;
        char* e = nullptr;
        const double v = strtod(b, &e);
        if (e == b) return ok = false;
        i += (size_t)(e - b);
        if (out) *out = v;
        return true;
    }
    // skips any value (nested at most kMaxDepth deep: a deeper file is malformed)
    static constexpr int kMaxDepth = 64;
    bool skip(int depth = 0) {
        ws();
        if (i >= t.size() || depth > kMaxDepth) return ok = false;
        const char c = t[i];
        if (c == '"') return str(nullptr);
        if (c == '{') {
            i++;
            if (eat('}')) return true;
            do {
                if (!str(nullptr) || !eat(':') || !skip(depth + 1)) return ok = false;
            } while (eat(','));
            if (eat('}')) return true;
            return ok = false;
        }
        if (c == '[') {
            i++;
            if (eat(']')) return true;
            do {
                if (!skip(depth + 1)) return ok = false;
            } while (eat(','));
            if (eat(']')) return true;
            return ok = false;
        }
        if (t.compare(i, 4, "true") == 0 || t.compare(i, 4, "null") == 0) {
            i += 4;
            return true;
        }
        if (t.compare(i, 5, "false") == 0) {
            i += 5;
            return true;
        }
        return num(nullptr);
    }
    bool entry(TuneEntry* e) {
        if (!eat('{')) return ok = false;
        if (eat('}')) return true;
        do {
            std::string k;
            if (!str(&k) || !eat(':')) return ok = false;
            double d = 0.0;
            if (k == "op") ok = str(&e->op);
            else if (k == "device") ok = str(&e->device);
            else if (k == "variant") ok = str(&e->variant);
            else if (k == "size_class") {
                ok = num(&d);
                e->size_class = (int)d;
            } else if (k == "ms") ok = num(&e->ms);
            else ok = skip();
            if (!ok) return false;
        } while (eat(','));
        if (eat('}')) return true;
        return ok = false;
    }
};

inline std::vector<TuneEntry> read_tune_cache(const std::string& path) {
    std::vector<TuneEntry> out;
    if (path.empty()) return out;
    FILE* f = fopen(path.c_str(), "rb");
    if (!f) return out;
    std::string text;
    char buf[4096];
    size_t n;
    while ((n = fread(buf, 1, sizeof(buf), f)) > 0 && text.size() < (16u << 20)) text.append(buf, n);
    fclose(f);
    JsonReader r(text);
    if (!r.eat('{') || r.eat('}')) return out;
    do {
        std::string k;
        if (!r.str(&k) || !r.eat(':')) return out;
        if (k == "entries") {
            if (!r.eat('[')) return out;
            if (r.eat(']')) continue;
            do {
                TuneEntry e;
                if (!r.entry(&e)) return out;
                if (!e.op.empty() && !e.variant.empty() && e.size_class >= 0 && e.size_class < 64) out.push_back(e);
            } while (r.eat(','));
            if (!r.eat(']')) return out;
        } else if (!r.skip()) {
            return out;
        }
    } while (r.eat(','));
    return out;
}

inline std::string json_escape(const std::string& x) {
    std::string r;
    for (char c : x) {
        if (c == '"' || c == '\\') r.push_back('\\');
        if ((unsigned char)c < 0x20) c = ' ';
        r.push_back(c);
    }
    return r;
}

// Creates the directories of `path` (mkdir -p of its parent).
inline void make_parent_dirs(const std::string& path) {
    for (size_t k = 1; k < path.size(); k++)
        if (path[k] == '/') mkdir(path.substr(0, k).c_str(), 0755);
}

// Writes the entries through a temporary file and a rename (a reader sees the
// old file or the new one, never a half-written one).  false on failure.
inline bool write_tune_cache(const std::string& path, const std::vector<TuneEntry>& v) {
    if (path.empty()) return false;
    make_parent_dirs(path);
    // a temporary name of this process and call: writers in other threads
    // or processes never share one (the last rename wins)
    static std::atomic<unsigned> seq{0};
    char suffix[64];
    snprintf(suffix, sizeof(suffix), ".tmp%ld.%u", (long)getpid(), seq.fetch_add(1));
    const std::string tmp = path + suffix;
    FILE* f = fopen(tmp.c_str(), "wb");
    if (!f) return false;
    fprintf(f, "{\"version\": 1, \"entries\": [");
    for (size_t k = 0; k < v.size(); k++)
        fprintf(f, "%s\n  {\"op\": \"%s\", \"device\": \"%s\", \"size_class\": %d, \"variant\": \"%s\", \"ms\": %.6g}",
                k ? "," : "", json_escape(v[k].op).c_str(), json_escape(v[k].device).c_str(), v[k].size_class,
                json_escape(v[k].variant).c_str(), v[k].ms);
    fprintf(f, "\n]}\n");
    const bool good = fflush(f) == 0;
    fclose(f);
    if (!good || rename(tmp.c_str(), path.c_str()) != 0) {
        unlink(tmp.c_str());
        return false;
    }
    return true;
}

}  // namespace pargo
