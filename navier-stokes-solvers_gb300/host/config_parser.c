/*
 * ns_config: flat dotted key/value configuration (drop-in for the reference's
 * src/common/config_parser.c:1-634, same API and semantics, own implementation).
 *
 *   INI   "[section]" then "key = value" -> "section.key"; '#' and ';' start
 *         comment lines; surrounding blanks are trimmed (:205-263).
 *   JSON  nested objects become dotted keys; strings (with \-escapes),
 *         true/false, null -> "" and numbers re-printed with %.15g (:364-480).
 *   Files load in order and later keys override earlier ones (:543-554); a
 *   ".json" extension (any case) selects JSON, anything else INI.
 *   Getters return the default when the key is missing or does not parse in
 *   full (:126-192); validate checks required keys, types, bounds and allowed
 *   strings (:556-634).
 */
#include "ns_config.h"

#include <ctype.h>
#include <errno.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#define NSC_KEY_MAX 256
#define NSC_VAL_MAX 512

static char *nsc_dup(const char *s) {
    const size_t n = strlen(s) + 1;
    char *d = (char *)malloc(n);
    if (d) memcpy(d, s, n);
    return d;
}

static int nsc_casecmp(const char *a, const char *b) {
    for (;; ++a, ++b) {
        const int ca = tolower((unsigned char)*a), cb = tolower((unsigned char)*b);
        if (ca != cb || !ca) return ca - cb;
    }
}

static void nsc_error(char *err, size_t n, const char *msg, const char *detail) {
    if (!err || !n) return;
    if (detail) snprintf(err, n, "%s: %s", msg, detail);
    else snprintf(err, n, "%s", msg);
}

/* strip leading and trailing white space in place */
static char *nsc_strip(char *s) {
    while (*s && isspace((unsigned char)*s)) ++s;
    char *e = s + strlen(s);
    while (e > s && isspace((unsigned char)e[-1])) --e;
    *e = '\0';
    return s;
}

void ns_config_init(NSConfig *c) {
    if (!c) return;
    c->entries = NULL;
    c->count = 0;
    c->capacity = 0;
}

void ns_config_free(NSConfig *c) {
    if (!c) return;
    for (size_t i = 0; i < c->count; ++i) {
        free(c->entries[i].key);
        free(c->entries[i].value);
    }
    free(c->entries);
    ns_config_init(c);
}

static NSConfigEntry *nsc_lookup(const NSConfig *c, const char *key) {
    if (!c || !key) return NULL;
    for (size_t i = 0; i < c->count; ++i)
        if (strcmp(c->entries[i].key, key) == 0) return &c->entries[i];
    return NULL;
}

int ns_config_set(NSConfig *c, const char *key, const char *value) {
    if (!c || !key || !value) return -1;
    NSConfigEntry *e = nsc_lookup(c, key);
    if (e) {
        char *v = nsc_dup(value);
        if (!v) return -1;
        free(e->value);
        e->value = v;
        return 0;
    }
    if (c->count == c->capacity) {
        const size_t cap = c->capacity ? 2 * c->capacity : 16;
        NSConfigEntry *ne = (NSConfigEntry *)realloc(c->entries, cap * sizeof(NSConfigEntry));
        if (!ne) return -1;
        c->entries = ne;
        c->capacity = cap;
    }
    char *k = nsc_dup(key), *v = nsc_dup(value);
    if (!k || !v) {
        free(k);
        free(v);
        return -1;
    }
    c->entries[c->count].key = k;
    c->entries[c->count].value = v;
    c->count++;
    return 0;
}

int ns_config_has_key(const NSConfig *c, const char *key) { return nsc_lookup(c, key) != NULL; }

const char *ns_config_get_string(const NSConfig *c, const char *key, const char *def) {
    const NSConfigEntry *e = nsc_lookup(c, key);
    return e ? e->value : def;
}

static int nsc_parse_long(const char *s, long *out) {
    if (!s || !*s) return 0;
    char *end = NULL;
    const long v = strtol(s, &end, 10);
    if (*end != '\0') return 0;
    *out = v;
    return 1;
}

static int nsc_parse_double(const char *s, double *out) {
    if (!s || !*s) return 0;
    char *end = NULL;
    const double v = strtod(s, &end);
    if (*end != '\0') return 0;
    *out = v;
    return 1;
}

/* 1 true, 0 false, -1 not a boolean */
static int nsc_parse_bool(const char *s) {
    if (!s || !*s) return -1;
    if (!nsc_casecmp(s, "true") || !nsc_casecmp(s, "yes") || !nsc_casecmp(s, "on") || !strcmp(s, "1")) return 1;
    if (!nsc_casecmp(s, "false") || !nsc_casecmp(s, "no") || !nsc_casecmp(s, "off") || !strcmp(s, "0")) return 0;
    return -1;
}

int ns_config_get_int(const NSConfig *c, const char *key, int def) {
    long v;
    const NSConfigEntry *e = nsc_lookup(c, key);
    return (e && nsc_parse_long(e->value, &v)) ? (int)v : def;
}

double ns_config_get_double(const NSConfig *c, const char *key, double def) {
    double v;
    const NSConfigEntry *e = nsc_lookup(c, key);
    return (e && nsc_parse_double(e->value, &v)) ? v : def;
}

int ns_config_get_bool(const NSConfig *c, const char *key, int def) {
    const NSConfigEntry *e = nsc_lookup(c, key);
    if (!e) return def;
    const int b = nsc_parse_bool(e->value);
    return b < 0 ? def : b;
}

/* ------------------------------------------------------------------- INI */

static int nsc_load_ini(NSConfig *c, FILE *fp, char *err, size_t errn) {
    char section[NSC_KEY_MAX] = "";
    char line[1024];
    while (fgets(line, sizeof(line), fp)) {
        char *s = nsc_strip(line);
        if (!*s || *s == '#' || *s == ';') continue;
        if (*s == '[') {
            char *close = strchr(s, ']');
            if (!close) {
                nsc_error(err, errn, "Malformed section header in INI file", s);
                return -1;
            }
            *close = '\0';
            snprintf(section, sizeof(section), "%s", nsc_strip(s + 1));
            continue;
        }
        char *eq = strchr(s, '=');
        if (!eq) {
            nsc_error(err, errn, "Malformed key-value line in INI file", s);
            return -1;
        }
        *eq = '\0';
        char keybuf[NSC_KEY_MAX], valbuf[NSC_VAL_MAX];
        snprintf(keybuf, sizeof(keybuf), "%s", s);
        snprintf(valbuf, sizeof(valbuf), "%s", eq + 1);
        const char *k = nsc_strip(keybuf), *v = nsc_strip(valbuf);
        char full[NSC_KEY_MAX];
        const int w = section[0] ? snprintf(full, sizeof(full), "%s.%s", section, k) : snprintf(full, sizeof(full), "%s", k);
        if (w < 0 || (size_t)w >= sizeof(full)) {
            nsc_error(err, errn, "Combined key too long", k);
            return -1;
        }
        if (ns_config_set(c, full, v) != 0) {
            nsc_error(err, errn, "Failed to store configuration key", full);
            return -1;
        }
    }
    return 0;
}

/* ------------------------------------------------------------------ JSON */

typedef struct {
    const char *p;
    NSConfig *c;
    char *err;
    size_t errn;
} nsc_json;

static void nsc_ws(nsc_json *j) {
    while (*j->p && isspace((unsigned char)*j->p)) ++j->p;
}

/* parse a JSON string at j->p (which points at '"'); returns malloc'd text */
static char *nsc_json_string(nsc_json *j) {
    nsc_ws(j);
    if (*j->p != '"') {
        nsc_error(j->err, j->errn, "Expected string in JSON configuration", NULL);
        return NULL;
    }
    ++j->p;
    size_t cap = 32, len = 0;
    char *buf = (char *)malloc(cap);
    if (!buf) return NULL;
    while (*j->p && *j->p != '"') {
        char ch = *j->p++;
        if (ch == '\\') {
            const char e = *j->p;
            if (!e) break;
            ++j->p;
            switch (e) {
                case 'b': ch = '\b'; break;
                case 'f': ch = '\f'; break;
                case 'n': ch = '\n'; break;
                case 'r': ch = '\r'; break;
                case 't': ch = '\t'; break;
                default: ch = e; break; /* \" \\ \/ and anything else map to themselves */
            }
        }
        if (len + 2 > cap) {
            cap *= 2;
            char *nb = (char *)realloc(buf, cap);
            if (!nb) {
                free(buf);
                return NULL;
            }
            buf = nb;
        }
        buf[len++] = ch;
    }
    if (*j->p != '"') {
        free(buf);
        nsc_error(j->err, j->errn, "Unterminated string in JSON configuration", NULL);
        return NULL;
    }
    ++j->p;
    buf[len] = '\0';
    return buf;
}

static int nsc_json_value(nsc_json *j, const char *key);

static int nsc_json_object(nsc_json *j, const char *prefix) {
    nsc_ws(j);
    if (*j->p != '{') {
        nsc_error(j->err, j->errn, "Expected '{' in JSON configuration", NULL);
        return -1;
    }
    ++j->p;
    nsc_ws(j);
    if (*j->p == '}') {
        ++j->p;
        return 0;
    }
    for (;;) {
        char *name = nsc_json_string(j);
        if (!name) return -1;
        nsc_ws(j);
        if (*j->p != ':') {
            free(name);
            nsc_error(j->err, j->errn, "Expected ':' in JSON key/value pair", NULL);
            return -1;
        }
        ++j->p;
        char full[NSC_KEY_MAX];
        const int w = (prefix && *prefix) ? snprintf(full, sizeof(full), "%s.%s", prefix, name)
                                          : snprintf(full, sizeof(full), "%s", name);
        free(name);
        if (w < 0 || (size_t)w >= sizeof(full)) {
            nsc_error(j->err, j->errn, "Combined JSON key too long", NULL);
            return -1;
        }
        if (nsc_json_value(j, full) != 0) return -1;
        nsc_ws(j);
        if (*j->p == ',') {
            ++j->p;
            continue;
        }
        if (*j->p == '}') {
            ++j->p;
            return 0;
        }
        nsc_error(j->err, j->errn, *j->p ? "Expected ',' or '}' in JSON object" : "Unexpected end of JSON content",
                  NULL);
        return -1;
    }
}

static int nsc_json_store(nsc_json *j, const char *key, const char *val) {
    if (ns_config_set(j->c, key, val) != 0) {
        nsc_error(j->err, j->errn, "Failed to store JSON value", key);
        return -1;
    }
    return 0;
}

static int nsc_json_value(nsc_json *j, const char *key) {
    nsc_ws(j);
    if (!*j->p) {
        nsc_error(j->err, j->errn, "Unexpected end of JSON value", NULL);
        return -1;
    }
    if (*j->p == '{') return nsc_json_object(j, key);
    if (*j->p == '"') {
        char *s = nsc_json_string(j);
        if (!s) return -1;
        const int r = nsc_json_store(j, key, s);
        free(s);
        return r;
    }
    static const struct {
        const char *lit;
        const char *val;
    } lits[] = {{"true", "true"}, {"false", "false"}, {"null", ""}};
    for (size_t i = 0; i < 3; ++i) {
        const size_t n = strlen(lits[i].lit);
        if (strncmp(j->p, lits[i].lit, n) == 0) {
            j->p += n;
            return nsc_json_store(j, key, lits[i].val);
        }
    }
    char *end = NULL;
    const double x = strtod(j->p, &end);
    if (end == j->p) {
        nsc_error(j->err, j->errn, "Invalid JSON value", key);
        return -1;
    }
    j->p = end;
    char num[64];
    snprintf(num, sizeof(num), "%.15g", x);
    return nsc_json_store(j, key, num);
}

static int nsc_load_json(NSConfig *c, FILE *fp, const char *path, char *err, size_t errn) {
    if (fseek(fp, 0, SEEK_END) != 0) {
        nsc_error(err, errn, "Failed to seek JSON configuration file", path);
        return -1;
    }
    const long len = ftell(fp);
    if (len < 0 || fseek(fp, 0, SEEK_SET) != 0) {
        nsc_error(err, errn, "Failed to determine JSON file size", path);
        return -1;
    }
    char *text = (char *)malloc((size_t)len + 1);
    if (!text) {
        nsc_error(err, errn, "Out of memory reading JSON configuration file", path);
        return -1;
    }
    if (fread(text, 1, (size_t)len, fp) != (size_t)len) {
        free(text);
        nsc_error(err, errn, "Failed to read JSON configuration file", path);
        return -1;
    }
    text[len] = '\0';
    nsc_json j = {text, c, err, errn};
    int r = nsc_json_object(&j, "");
    if (r == 0) {
        nsc_ws(&j);
        if (*j.p) {
            nsc_error(err, errn, "Unexpected trailing data in JSON file", NULL);
            r = -1;
        }
    }
    free(text);
    return r;
}

int ns_config_load_files(NSConfig *c, const char **paths, size_t count, char *err, size_t errn) {
    if (!c || (!paths && count > 0)) {
        nsc_error(err, errn, "Invalid arguments to ns_config_load_files", NULL);
        return -1;
    }
    for (size_t i = 0; i < count; ++i) {
        const char *dot = strrchr(paths[i], '.');
        const int json = dot && nsc_casecmp(dot, ".json") == 0;
        FILE *fp = fopen(paths[i], json ? "rb" : "r");
        if (!fp) {
            nsc_error(err, errn, json ? "Failed to open JSON configuration file" : "Failed to open INI configuration file",
                      strerror(errno));
            return -1;
        }
        const int r = json ? nsc_load_json(c, fp, paths[i], err, errn) : nsc_load_ini(c, fp, err, errn);
        fclose(fp);
        if (r != 0) return -1;
    }
    return 0;
}

int ns_config_validate(const NSConfig *c, const NSConfigSchemaEntry *schema, size_t n, char *err, size_t errn) {
    if (!c || !schema) {
        nsc_error(err, errn, "Invalid arguments to ns_config_validate", NULL);
        return -1;
    }
    for (size_t i = 0; i < n; ++i) {
        const NSConfigSchemaEntry *s = &schema[i];
        const NSConfigEntry *e = nsc_lookup(c, s->key);
        if (!e) {
            if (s->required) {
                nsc_error(err, errn, "Missing required configuration key", s->key);
                return -1;
            }
            continue;
        }
        const char *v = e->value;
        switch (s->type) {
            case NS_CONFIG_VALUE_STRING:
                if (s->allowed_values && s->allowed_count > 0) {
                    size_t a = 0;
                    while (a < s->allowed_count && nsc_casecmp(v, s->allowed_values[a]) != 0) ++a;
                    if (a == s->allowed_count) {
                        nsc_error(err, errn, "Configuration string value not permitted", s->key);
                        return -1;
                    }
                }
                break;
            case NS_CONFIG_VALUE_INT:
            case NS_CONFIG_VALUE_DOUBLE: {
                double x;
                long l;
                const int is_int = (s->type == NS_CONFIG_VALUE_INT);
                if (is_int ? !nsc_parse_long(v, &l) : !nsc_parse_double(v, &x)) {
                    nsc_error(err, errn, is_int ? "Configuration key expects integer value"
                                                : "Configuration key expects numeric value",
                              s->key);
                    return -1;
                }
                if (is_int) x = (double)l;
                if (s->has_min && x < s->min_value) {
                    nsc_error(err, errn, is_int ? "Configuration integer below minimum" : "Configuration value below minimum",
                              s->key);
                    return -1;
                }
                if (s->has_max && x > s->max_value) {
                    nsc_error(err, errn, is_int ? "Configuration integer above maximum" : "Configuration value above maximum",
                              s->key);
                    return -1;
                }
                break;
            }
            case NS_CONFIG_VALUE_BOOL:
                if (nsc_parse_bool(v) < 0) {
                    nsc_error(err, errn, "Configuration key expects boolean value", s->key);
                    return -1;
                }
                break;
        }
    }
    return 0;
}
