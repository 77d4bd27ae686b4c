// psdata.cpp -- the host particle store (psdata), the .conf section reader
// and logging of libsph_gb300.so.
//
// The store keeps the reference's layout bit for bit, because the Python
// interface and every kernel address fields by those offsets:
//   - the field-spec grammar `name | dims | type | values` with `#` comment
//     lines (src/build_psdata.c:184-326, :585-613);
//   - the neighbour-grid arrays appended after the conf's fields
//     (build_psdata.c:40-183);
//   - fields reordered double > float > unsigned int > rest, keeping conf
//     order within each group (build_psdata.c:519-576);
//   - each field aligned to its first-dimension tuple (entry size x dims[0]
//     when it has more than one dimension), computed with the same unsigned
//     wrap-around for the first field (build_psdata.c:373-382).
// The parser is written afresh (no strtok); the tests pin its output
// against the reference's own builder.
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <memory>
#include <string>
#include <vector>

#include "sph_gb300.h"
#include "sph_internal.h"

// ---------------------------------------------------------------------------
// logging (src/note.c:7-33)

static unsigned int g_loglevel = 1;

extern "C" void set_log_level(unsigned int loglevel) { g_loglevel = loglevel; }

extern "C" void note(unsigned int level, const char *fmt, ...) {
    if (level < g_loglevel) return;
    va_list args;
    va_start(args, fmt);
    vprintf(fmt, args);
    va_end(args);
    fflush(stdout);
}

// ---------------------------------------------------------------------------
// type strings (src/stringly.c:5-60)

namespace {

struct TypeInfo {
    const char *name;
    FieldType type;
    unsigned size;
};
const TypeInfo kTypes[] = {
    {"char", T_CHAR, 1},      {"unsigned int", T_UINT, 4}, {"uint", T_UINT, 4},
    {"int", T_INT, 4},        {"float", T_FLOAT32, 4},     {"float32", T_FLOAT32, 4},
    {"double", T_FLOAT64, 8}, {"float64", T_FLOAT64, 8},
};

const TypeInfo *find_type(const std::string &t) {
    for (const TypeInfo &ti : kTypes)
        if (t == ti.name) return &ti;
    return nullptr;
}

// One parsed conf line.
struct FieldSpec {
    std::string name;
    std::vector<unsigned> dims;
    std::string type;
    std::vector<unsigned char> value;  // raw bytes of the given default values
};

// Tokens of `s` separated by any character of `delims`, empty tokens
// dropped (the splitting rule of the reference's strtok loops).
std::vector<std::string> split(const std::string &s, const char *delims) {
    std::vector<std::string> out;
    size_t i = 0, n = s.size();
    while (i < n) {
        while (i < n && strchr(delims, s[i])) ++i;
        size_t j = i;
        while (j < n && !strchr(delims, s[j])) ++j;
        if (j > i) out.push_back(s.substr(i, j - i));
        i = j;
    }
    return out;
}

const FieldSpec *find_spec(const std::vector<FieldSpec> &list, const std::string &name) {
    for (const FieldSpec &f : list)
        if (f.name == name) return &f;
    return nullptr;
}

// get_value, build_psdata.c:29-37: the first 4 bytes of a named field's
// default value read as unsigned; UINT_MAX when the field is absent.  A
// field without a value (the reference dereferences NULL there) reads 0.
unsigned value_of(const std::vector<FieldSpec> &list, const std::string &name) {
    const FieldSpec *f = find_spec(list, name);
    if (!f) return 0xFFFFFFFFu;
    if (f->value.size() < 4) return 0;
    unsigned v;
    memcpy(&v, f->value.data(), 4);
    return v;
}

// create_psdata_field_spec, build_psdata.c:184-326
bool parse_line(const std::string &line, const std::vector<FieldSpec> &list, FieldSpec *out) {
    const size_t kMaxDims = 5, kMaxType = 64, kMaxValue = 256;
    std::vector<std::string> segments = split(line, "|");
    for (size_t seg = 0; seg < segments.size(); ++seg) {
        std::vector<std::string> words = split(segments[seg], ", ");
        for (size_t w = 0; w < words.size(); ++w) {
            const std::string &word = words[w];
            if (seg == 0) {
                if (w == 0) out->name = word;
            } else if (seg == 1) {
                if (out->dims.size() == kMaxDims) {
                    note(1, "%s: Over maximum number of dimensions\n", out->name.c_str());
                    break;
                }
                unsigned dim = (unsigned)strtol(word.c_str(), nullptr, 0);
                if (dim == 0 && !list.empty()) {
                    dim = value_of(list, word);
                    if (dim == 0xFFFFFFFFu) dim = 0;
                }
                out->dims.push_back(dim);
            } else if (seg == 2) {
                size_t add = out->type.size() + word.size() + 1;
                if (add >= kMaxType) {
                    note(1, "%s: Over maximum type string length\n", out->name.c_str());
                    break;
                }
                if (!out->type.empty()) out->type += ' ';
                out->type += word;
            } else if (seg == 3) {
                // Only these four spellings take default values
                // (build_psdata.c:257-293).
                unsigned char buf[8];
                size_t sz = 0;
                if (out->type == "double") {
                    double v = strtod(word.c_str(), nullptr);
                    memcpy(buf, &v, sz = 8);
                } else if (out->type == "float") {
                    float v = strtof(word.c_str(), nullptr);
                    memcpy(buf, &v, sz = 4);
                } else if (out->type == "unsigned int") {
                    unsigned v = (unsigned)strtol(word.c_str(), nullptr, 0);
                    memcpy(buf, &v, sz = 4);
                } else if (out->type == "int") {
                    int v = (int)strtol(word.c_str(), nullptr, 0);
                    memcpy(buf, &v, sz = 4);
                }
                if (sz == 0) continue;
                if (out->value.size() + sz > kMaxValue) {
                    note(1, "%s: Over maximum default value length\n", out->name.c_str());
                    break;
                }
                out->value.insert(out->value.end(), buf, buf + sz);
            }
        }
    }
    if (out->name.empty()) {
        sph_set_error("psdata: line without a field name: '%s'", line.c_str());
        return false;
    }
    return true;
}

FieldSpec grid_field(const char *name, std::vector<unsigned> dims) {
    FieldSpec f;
    f.name = name;
    f.dims = dims;
    f.type = "unsigned int";
    return f;
}

// add_grid_arrays, build_psdata.c:40-183
bool add_grid_arrays(std::vector<FieldSpec> &list) {
    const FieldSpec *h = find_spec(list, "smoothingradius");
    const FieldSpec *gb = find_spec(list, "gridbounds");
    if (!h || !gb) {
        sph_set_error("psdata: smoothingradius and gridbounds fields are required");
        return false;
    }
    if (h->value.empty()) {
        note(1, "No value for smoothingradius\n");
        return true;
    }
    bool h_double = h->type == "double";
    if (!h_double && h->type != "float") {
        sph_set_error("psdata: smoothingradius must be float or double");
        return false;
    }
    if (gb->value.empty()) {
        note(1, "No value for gridbounds\n");
        return true;
    }
    bool gb_double = gb->type == "double";
    if ((!gb_double && gb->type != "float") || gb_double != h_double) {
        sph_set_error("psdata: gridbounds must have smoothingradius's type");
        return false;
    }
    unsigned pnum = value_of(list, "pnum");
    if (pnum == 0xFFFFFFFFu) {
        note(1, "No value for pnum\n");
        return true;
    }
    unsigned res[3];
    size_t need = (h_double ? 8 : 4) * 6;
    std::vector<unsigned char> bounds(gb->value);
    bounds.resize(need > bounds.size() ? need : bounds.size(), 0);
    for (int a = 0; a < 3; ++a) {
        double extent, hh;
        if (h_double) {
            double b0, b1;
            memcpy(&b0, bounds.data() + 16 * a, 8);
            memcpy(&b1, bounds.data() + 16 * a + 8, 8);
            memcpy(&hh, h->value.data(), 8);
            extent = fabs(b1 - b0);
        } else {
            // fabs() of the float difference is taken in double, and the
            // division by the float radius too (build_psdata.c:96-98)
            float b0, b1, hf;
            memcpy(&b0, bounds.data() + 8 * a, 4);
            memcpy(&b1, bounds.data() + 8 * a + 4, 4);
            memcpy(&hf, h->value.data(), 4);
            extent = fabs((double)(b1 - b0));
            hh = (double)hf;
        }
        double r = extent / hh;
        res[a] = (r > 0 && r < 4294967296.0) ? (unsigned)r : 0u;
    }
    FieldSpec gridres = grid_field("gridres", {3});
    gridres.value.resize(12);
    memcpy(gridres.value.data(), res, 12);
    list.push_back(gridres);
    list.push_back(grid_field("gridcell", {pnum}));
    list.push_back(grid_field("gridcount", {res[0], res[1], res[2]}));
    list.push_back(grid_field("celloffset", {res[0], res[1], res[2]}));
    list.push_back(grid_field("cellparticles", {pnum}));
    return true;
}

// sort_field_spec_list_by_type_size_descending, build_psdata.c:519-576
std::vector<FieldSpec> sort_by_type(const std::vector<FieldSpec> &list) {
    static const char *order[] = {"double", "float", "unsigned int"};
    std::vector<FieldSpec> out;
    std::vector<bool> used(list.size(), false);
    for (const char *t : order)
        for (size_t i = 0; i < list.size(); ++i)
            if (!used[i] && list[i].type == t) { out.push_back(list[i]); used[i] = true; }
    for (size_t i = 0; i < list.size(); ++i)
        if (!used[i]) out.push_back(list[i]);
    return out;
}

template <typename T>
T *alloc_copy(const std::vector<T> &v) {
    T *p = (T *)malloc((v.size() ? v.size() : 1) * sizeof(T));
    if (!v.empty()) memcpy(p, v.data(), v.size() * sizeof(T));
    return p;
}

// populate_psdata, build_psdata.c:327-486
bool populate(psdata *d, const std::vector<FieldSpec> &list) {
    unsigned nf = (unsigned)list.size();
    std::vector<unsigned> names_off(nf), ndims(nf), dims_off(nf), entry(nf), sizes(nf), offsets(nf);
    std::vector<unsigned> dims;
    std::string names;
    uint64_t data_size = 0;
    for (unsigned f = 0; f < nf; ++f) {
        const FieldSpec &fs = list[f];
        names_off[f] = (unsigned)names.size();
        names += fs.name;
        names += '\0';
        ndims[f] = (unsigned)fs.dims.size();
        dims_off[f] = (unsigned)dims.size();
        dims.insert(dims.end(), fs.dims.begin(), fs.dims.end());
        const TypeInfo *ti = find_type(fs.type);
        entry[f] = ti ? ti->size : 0;
        uint64_t sz = entry[f];
        for (unsigned dm : fs.dims) sz *= dm;
        sizes[f] = (unsigned)sz;
        uint64_t tuplet = fs.dims.size() > 1 ? (uint64_t)entry[f] * fs.dims[0] : entry[f];
        if (tuplet == 0) {
            sph_set_error("psdata: field '%s' has a zero-sized entry (unknown type '%s' or zero first dimension)",
                          fs.name.c_str(), fs.type.c_str());
            return false;
        }
        // (data_size - 1) wraps to 2^64-1 for the first field, exactly as the
        // reference's size_t arithmetic does; the result is kept in 32 bits.
        offsets[f] = (unsigned)(tuplet * ((data_size - 1) / tuplet + 1));
        data_size = (uint64_t)offsets[f] + sizes[f];
    }
    if (data_size > 0xFFFFFFFFull) {
        sph_set_error("psdata: store of %llu bytes exceeds the 32-bit offsets of the format",
                      (unsigned long long)data_size);
        return false;
    }
    d->num_fields = nf;
    char *nm = (char *)malloc(names.size() ? names.size() : 1);
    memcpy(nm, names.data(), names.size());
    d->names = nm;
    d->names_offsets = alloc_copy(names_off);
    d->dimensions = alloc_copy(dims);
    d->num_dimensions = alloc_copy(ndims);
    d->dimensions_offsets = alloc_copy(dims_off);
    d->entry_sizes = alloc_copy(entry);
    d->data_sizes = alloc_copy(sizes);
    d->data_offsets = alloc_copy(offsets);
    d->data = calloc(data_size ? data_size : 1, 1);
    d->data_ptrs = (DataPtr *)malloc((nf ? nf : 1) * sizeof(DataPtr));
    for (unsigned f = 0; f < nf; ++f) {
        const FieldSpec &fs = list[f];
        // The reference copies data_sizes[f] bytes from the default value;
        // only the bytes actually given are copied here, the rest stay 0.
        size_t ncopy = fs.value.size() < sizes[f] ? fs.value.size() : sizes[f];
        if (ncopy) memcpy((char *)d->data + offsets[f], fs.value.data(), ncopy);
        const TypeInfo *ti = find_type(fs.type);
        d->data_ptrs[f].type = ti ? ti->type : T_CHAR;
        d->data_ptrs[f].ptr = (char *)d->data + offsets[f];
    }
    d->num_host_fields = 0;
    d->host_names = nullptr;
    d->host_data = nullptr;
    d->host_data_size = nullptr;
    return true;
}

}  // namespace

// ---------------------------------------------------------------------------
// store ABI

extern "C" void build_psdata_from_string(psdata *data, const char *string) {
    memset(data, 0, sizeof(*data));
    std::vector<FieldSpec> list;
    std::vector<std::string> lines = split(string ? string : "", "\n");
    for (const std::string &line : lines) {
        if (!line.empty() && line[0] == '#') continue;
        FieldSpec fs;
        if (!parse_line(line, list, &fs)) { sph_fail(); return; }
        list.push_back(fs);
    }
    if (!add_grid_arrays(list) || !populate(data, sort_by_type(list))) {
        memset(data, 0, sizeof(*data));
        sph_fail();
    }
}

extern "C" void build_psdata(psdata *data, const char *path) {
    FILE *f = fopen(path, "rb");
    if (!f) {
        note(1, "Could not read file %s\n", path);
        sph_set_error("build_psdata: could not read file %s", path);
        sph_fail();
        return;
    }
    fseek(f, 0, SEEK_END);
    long end = ftell(f);
    fseek(f, 0, SEEK_SET);
    std::string s((size_t)(end > 0 ? end : 0), '\0');
    if (end > 0 && fread(&s[0], 1, (size_t)end, f) != (size_t)end) s.clear();
    fclose(f);
    // the reference overwrites the file's last byte with the terminator
    // (build_psdata.c:631)
    if (!s.empty()) s.pop_back();
    build_psdata_from_string(data, s.c_str());
}

// display_psdata / display_entry, particle_system.c:38-82 (level-2 notes)
static void display_entry(const psdata &d, size_t off, size_t size) {
    if (size == 8) note(2, "%g, ", *(const double *)((const char *)d.data + off));
    else if (size == 4) note(2, "%u, ", *(const unsigned *)((const char *)d.data + off));
}

extern "C" void display_psdata(psdata d, const char *const *mask) {
    if (mask != nullptr) return;
    for (unsigned f = 0; f < d.num_fields; ++f) {
        note(2, "%s:\n\n", d.names + d.names_offsets[f]);
        const unsigned *dm = d.dimensions + d.dimensions_offsets[f];
        unsigned nd = d.num_dimensions[f], es = d.entry_sizes[f];
        size_t off = d.data_offsets[f];
        if (nd == 1) {
            for (unsigned i = 0; i < dm[0]; ++i) display_entry(d, off + (size_t)i * es, es);
        } else if (nd == 2) {
            for (unsigned i = 0; i < dm[1]; ++i) {
                for (unsigned j = 0; j < dm[0]; ++j) display_entry(d, off + ((size_t)i * dm[0] + j) * es, es);
                note(2, "\n");
            }
        } else if (nd == 3) {
            for (unsigned i = 0; i < dm[2]; ++i) {
                for (unsigned j = 0; j < dm[1]; ++j) {
                    for (unsigned k = 0; k < dm[0]; ++k)
                        display_entry(d, off + ((size_t)i * dm[1] * dm[0] + (size_t)j * dm[0] + k) * es, es);
                    note(2, "\n");
                }
                note(2, "\n");
            }
        }
        note(2, "\n\n");
    }
}

// particle_system.c:84-91
extern "C" int get_field_psdata(psdata d, const char *name) {
    for (unsigned i = 0; i < d.num_fields; ++i)
        if (strcmp(d.names + d.names_offsets[i], name) == 0) return (int)i;
    return -1;
}

// particle_system.c:93-97
extern "C" void set_field_psdata(psdata *d, const char *name, void *field, unsigned size, unsigned offset) {
    int i = get_field_psdata(*d, name);
    if (i != -1) memcpy((char *)d->data + d->data_offsets[i] + offset, field, size);
}

// particle_system.c:99-112
extern "C" unsigned psdata_names_size(psdata d) {
    if (d.num_fields == 0) return 0;
    const char *last = d.names + d.names_offsets[d.num_fields - 1];
    return d.names_offsets[d.num_fields - 1] + (unsigned)strlen(last) + 1;
}
extern "C" unsigned psdata_dimensions_size(psdata d) {
    if (d.num_fields == 0) return 0;
    unsigned nf = d.num_fields;
    return (d.dimensions_offsets[nf - 1] + d.num_dimensions[nf - 1]) * (unsigned)sizeof(unsigned);
}
extern "C" unsigned psdata_data_size(psdata d) {
    if (d.num_fields == 0) return 0;
    return d.data_offsets[d.num_fields - 1] + d.data_sizes[d.num_fields - 1];
}

// particle_system.c:116-164
extern "C" int create_host_field_psdata(psdata *d, const char *name, void *field, unsigned size) {
    unsigned n = d->num_host_fields + 1;
    d->host_names = (char **)realloc(d->host_names, n * sizeof(char *));
    d->host_data = (void **)realloc(d->host_data, n * sizeof(void *));
    d->host_data_size = (unsigned *)realloc(d->host_data_size, n * sizeof(unsigned));
    char *copy = (char *)malloc(strlen(name) + 1);
    strcpy(copy, name);
    d->host_names[n - 1] = copy;
    d->host_data[n - 1] = field;
    d->host_data_size[n - 1] = size;
    d->num_host_fields = n;
    return (int)(n - 1);
}
extern "C" int get_host_field_psdata(psdata *d, const char *name) {
    for (unsigned i = 0; i < d->num_host_fields; ++i)
        if (strcmp(d->host_names[i], name) == 0) return (int)i;
    return -1;
}

// particle_system.c:218-255
extern "C" void free_psdata(psdata *d) {
    free((void *)d->names);
    free(d->names_offsets);
    free(d->dimensions);
    free(d->num_dimensions);
    free(d->dimensions_offsets);
    free(d->entry_sizes);
    free(d->data);
    free(d->data_sizes);
    free(d->data_offsets);
    free(d->data_ptrs);
    for (unsigned i = 0; i < d->num_host_fields; ++i) {
        free(d->host_data[i]);
        free(d->host_names[i]);
    }
    free(d->host_names);
    free(d->host_data);
    free(d->host_data_size);
    memset(d, 0, sizeof(*d));
    note(1, "freed host data\n");
}

// ---------------------------------------------------------------------------
// config sections (src/config.c:19-106).  A file splits into `$title` lines,
// each followed by its section's text up to the next `$`.  The reference
// cuts the file with the C library's tokenizer, and its rules decide what a
// malformed file gives, so the same rules are kept here (take() below):
//   - text before the first `$` is skipped;
//   - a title is the run after `$` up to the end of its line; a `$` at the
//     very start of the file keeps any newlines right after it as the
//     title's start, elsewhere empty lines before a title are skipped;
//   - a section's text runs to the next `$`, skipping `$`s in front of it,
//     so a section with no text takes the next `$title` line and text as
//     its own;
//   - a title with no text after it is dropped;
//   - at most 8 sections are kept, counted across loads until
//     unload_config (a second load_config adds to the first's sections and
//     a title found in both returns the first's text).

namespace {
// The files read since the last unload_config, split in place; the
// sections point into them.
std::vector<std::unique_ptr<std::string>> g_conf_files;
std::vector<std::pair<const char *, const char *>> g_sections;  // title, text

// The next token of the text at *at: skip characters of `seps`, take the
// run up to the next one, end it in place with a NUL and move *at past it.
// nullptr when only separators are left.
char *take(char **at, const char *seps) {
    char *q = *at + strspn(*at, seps);
    if (!*q) {
        *at = q;
        return nullptr;
    }
    char *e = q + strcspn(q, seps);
    if (*e) *e++ = '\0';
    *at = e;
    return q;
}
}  // namespace

extern "C" int load_config(const char *path) {
    FILE *f = fopen(path, "rb");
    if (!f) {
        note(2, "Could not read file %s\n", path);
        return 1;
    }
    fseek(f, 0, SEEK_END);
    long end = ftell(f);
    fseek(f, 0, SEEK_SET);
    auto text = std::make_unique<std::string>((size_t)(end > 0 ? end : 0), '\0');
    if (end > 0 && fread(&(*text)[0], 1, (size_t)end, f) != (size_t)end) text->clear();
    fclose(f);
    g_conf_files.push_back(std::move(text));
    char *buf = &(*g_conf_files.back())[0];  // NUL-terminated by std::string
    char *at = buf, *title;
    if (buf[0] == '$') {
        at = buf + 1;
        take(&at, "\n");
        title = buf + 1;
    } else {
        take(&at, "$");
        title = take(&at, "\n");
    }
    while (title && g_sections.size() < 8) {
        char *body = take(&at, "$");
        if (!body) break;
        g_sections.emplace_back(title, body);
        title = take(&at, "\n");
    }
    return 0;
}

extern "C" const char *get_config_section(const char *heading) {
    for (auto &s : g_sections)
        if (!strcmp(s.first, heading)) return s.second;
    return nullptr;
}

extern "C" void unload_config(void) {
    g_sections.clear();
    g_conf_files.clear();
}
