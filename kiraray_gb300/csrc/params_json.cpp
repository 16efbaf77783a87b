// Pass parameters from JSON, as WavefrontPathTracer::from_json reads them
// (src/render/wavefront/integrator.h:85-103): the keys "nee",
// "enable_medium", "max_depth", "rr", "enable_clamp" and "clamp_max" with the
// reference's defaults, plus this library's "spp", "seed" and
// "independent_samples".  Keys that are absent keep their defaults and other
// keys are ignored, as the reference's `j.value(key, default)` lookups do; a
// key of the wrong type or malformed JSON is an error (the reference's json
// library throws there).
//
// The parser is a small recursive-descent reader of RFC 8259 JSON: the
// top-level value must be an object; nested values are parsed and skipped.
#include <cctype>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <string>

#include "internal.h"

namespace {

struct Reader {
    const char *p;
    const char *err = nullptr;

    void ws() {
        while (*p == ' ' || *p == '\t' || *p == '\n' || *p == '\r') ++p;
    }
    bool fail(const char *what) {
        if (!err) err = what;
        return false;
    }
    bool lit(const char *word) {
        size_t n = std::strlen(word);
        if (std::strncmp(p, word, n) != 0) return fail("unknown literal");
        p += n;
        return true;
    }
    bool string(std::string *out) {
        if (*p != '"') return fail("expected a string");
        ++p;
        while (*p && *p != '"') {
            char c = *p++;
            if ((unsigned char)c < 0x20) return fail("control character in a string");
            if (c == '\\') {
                char e = *p++;
                switch (e) {
                    case '"': case '\\': case '/': c = e; break;
                    case 'b': c = '\b'; break;
                    case 'f': c = '\f'; break;
                    case 'n': c = '\n'; break;
                    case 'r': c = '\r'; break;
                    case 't': c = '\t'; break;
                    case 'u':
                        for (int k = 0; k < 4; ++k)
                            if (!std::isxdigit((unsigned char)*p++)) return fail("bad \\u escape");
                        c = '?';   // key names here are ASCII; other code points are kept as '?'
                        break;
                    default: return fail("bad escape");
                }
            }
            if (out) out->push_back(c);
        }
        if (*p != '"') return fail("unterminated string");
        ++p;
        return true;
    }
    bool number(double *out) {
        const char *s = p;
        if (*p == '-') ++p;
        if (!std::isdigit((unsigned char)*p)) return fail("bad number");
        if (*p == '0') ++p;
        else while (std::isdigit((unsigned char)*p)) ++p;
        if (*p == '.') {
            ++p;
            if (!std::isdigit((unsigned char)*p)) return fail("bad number");
            while (std::isdigit((unsigned char)*p)) ++p;
        }
        if (*p == 'e' || *p == 'E') {
            ++p;
            if (*p == '+' || *p == '-') ++p;
            if (!std::isdigit((unsigned char)*p)) return fail("bad number");
            while (std::isdigit((unsigned char)*p)) ++p;
        }
        if (out) *out = std::strtod(std::string(s, p).c_str(), nullptr);
        return true;
    }
    // kind: 0 null, 1 bool, 2 number, 3 string, 4 array, 5 object
    bool value(int depth, int *kind, double *num, bool *flag) {
        if (depth > 64) return fail("nesting too deep");
        ws();
        switch (*p) {
            case '{': {
                *kind = 5;
                ++p;
                ws();
                if (*p == '}') { ++p; return true; }
                while (true) {
                    ws();
                    if (!string(nullptr)) return false;
                    ws();
                    if (*p++ != ':') return fail("expected ':'");
                    int k; double d; bool b;
                    if (!value(depth + 1, &k, &d, &b)) return false;
                    ws();
                    if (*p == ',') { ++p; continue; }
                    if (*p == '}') { ++p; return true; }
                    return fail("expected ',' or '}'");
                }
            }
            case '[': {
                *kind = 4;
                ++p;
                ws();
                if (*p == ']') { ++p; return true; }
                while (true) {
                    int k; double d; bool b;
                    if (!value(depth + 1, &k, &d, &b)) return false;
                    ws();
                    if (*p == ',') { ++p; continue; }
                    if (*p == ']') { ++p; return true; }
                    return fail("expected ',' or ']'");
                }
            }
            case '"': *kind = 3; return string(nullptr);
            case 't': *kind = 1; *flag = true; return lit("true");
            case 'f': *kind = 1; *flag = false; return lit("false");
            case 'n': *kind = 0; return lit("null");
            default: *kind = 2; return number(num);
        }
    }
};

enum Type { kBool, kInt, kFloat, kUint };

struct Key {
    const char *name;
    Type type;
};

const Key kKeys[] = {{"nee", kBool},          {"enable_medium", kBool}, {"max_depth", kInt},
                     {"rr", kFloat},          {"enable_clamp", kBool},  {"clamp_max", kFloat},
                     {"spp", kInt},           {"seed", kUint},          {"independent_samples", kBool}};

void assign(krr_wf_params *p, int key, double v) {
    switch (key) {
        case 0: p->nee = v != 0; break;
        case 1: p->enable_medium = v != 0; break;
        case 2: p->max_depth = (int32_t)v; break;
        case 3: p->rr = (float)v; break;
        case 4: p->enable_clamp = v != 0; break;
        case 5: p->clamp_max = (float)v; break;
        case 6: p->spp = (int32_t)v; break;
        case 7: p->seed = (uint32_t)v; break;
        case 8: p->independent_samples = v != 0; break;
    }
}

}  // namespace

// Parses the pass parameters of `json` over the defaults (or over *inout
// when `over_current`).
static int params_from_json(const char *json, krr_wf_params *inout, bool over_current) {
    if (!json || !inout) return krr::fail(KRR_ERR_INVALID_ARGUMENT, "NULL argument");
    krr_wf_params p;
    if (over_current) p = *inout;
    else krr_wf_params_default(&p);
    Reader r{json};
    r.ws();
    if (*r.p != '{') return krr::fail(KRR_ERR_INVALID_ARGUMENT, "pass parameters: expected a JSON object");
    ++r.p;
    r.ws();
    bool first = true;
    while (*r.p != '}') {
        if (!first) {
            if (*r.p != ',') return krr::fail(KRR_ERR_INVALID_ARGUMENT, "pass parameters: expected ','");
            ++r.p;
            r.ws();
        }
        first = false;
        std::string key;
        if (!r.string(&key)) break;
        r.ws();
        if (*r.p++ != ':') { r.fail("expected ':'"); break; }
        int kind = -1;
        double num = 0;
        bool flag = false;
        if (!r.value(1, &kind, &num, &flag)) break;
        r.ws();
        for (int k = 0; k < (int)(sizeof(kKeys) / sizeof(kKeys[0])); ++k) {
            if (key != kKeys[k].name) continue;
            const Type t = kKeys[k].type;
            if (t == kBool && kind == 1) assign(&p, k, flag ? 1.0 : 0.0);
            else if (t == kBool && kind == 2 && (num == 0 || num == 1)) assign(&p, k, num);
            else if (t == kFloat && kind == 2) assign(&p, k, num);
            else if ((t == kInt || t == kUint) && kind == 2 && num == std::floor(num) &&
                     num >= (t == kUint ? 0.0 : -2147483648.0) &&
                     num <= (t == kUint ? 4294967295.0 : 2147483647.0))
                assign(&p, k, num);
            else
                return krr::fail(KRR_ERR_INVALID_ARGUMENT, "pass parameter \"%s\" has the wrong type",
                                 kKeys[k].name);
        }
    }
    if (r.err) return krr::fail(KRR_ERR_INVALID_ARGUMENT, "pass parameters: malformed JSON (%s)", r.err);
    ++r.p;
    r.ws();
    if (*r.p) return krr::fail(KRR_ERR_INVALID_ARGUMENT, "pass parameters: text after the JSON object");
    if (p.max_depth < 0 || p.spp < 1)
        return krr::fail(KRR_ERR_INVALID_ARGUMENT, "pass parameters: max_depth >= 0 and spp >= 1");
    *inout = p;
    return KRR_OK;
}

extern "C" int krr_wf_params_from_json(const char *json, krr_wf_params *out) {
    return params_from_json(json, out, false);
}

extern "C" int krr_wf_create_json(const char *params_json, krr_wf **out) {
    krr_wf_params p;
    KRR_TRY(params_from_json(params_json ? params_json : "{}", &p, false));
    return krr_wf_create(&p, out);
}

extern "C" int krr_wf_set_params_json(krr_wf *wf, const char *params_json) {
    KRR_CHECK_ARG(wf && params_json, "NULL argument");
    krr_wf_params p;
    KRR_TRY(krr_wf_get_params(wf, &p));
    KRR_TRY(params_from_json(params_json, &p, true));
    return krr_wf_set_params(wf, &p);
}
