// Versioned plan file: one symgb_plan_desc with its index, output-index and
// constant tables, written once and reloaded without running the front end.
//
// The reference writes only the three tables, as raw arrays named
// indexData / constData / outIndexData (src/Utilities.hpp:156-161), and bakes
// everything else into the generated source.  This file carries the whole
// plan: header (magic, format version, byte-order mark), sizes, argument and
// output ranges, every kernel (offsets, row counts, level, post-order
// template, access table), the tables, and an FNV-1a 64 checksum of all
// preceding bytes.  Little-endian fixed-width fields throughout.
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "symgb.h"

namespace {

constexpr char kMagic[8] = {'S', 'Y', 'M', 'G', 'B', 'P', 'L', 'N'};
constexpr std::uint32_t kVersion = 1;
constexpr std::uint32_t kByteOrder = 0x01020304u;

thread_local std::string g_planError;

int planFail(const std::string& msg) {
    g_planError = msg;
    return SYMGB_ERR_ARGUMENT;
}

struct Writer {
    std::vector<unsigned char> buf;
    template <class T>
    void put(const T& v) {
        const auto* p = reinterpret_cast<const unsigned char*>(&v);
        buf.insert(buf.end(), p, p + sizeof(T));
    }
    template <class T>
    void putArray(const T* p, std::size_t n) {
        if (n == 0) return;
        const auto* b = reinterpret_cast<const unsigned char*>(p);
        buf.insert(buf.end(), b, b + n * sizeof(T));
    }
};

struct Reader {
    const unsigned char* p;
    std::size_t left;
    bool ok = true;
    template <class T>
    T get() {
        T v{};
        if (left < sizeof(T)) {
            ok = false;
            return v;
        }
        std::memcpy(&v, p, sizeof(T));
        p += sizeof(T);
        left -= sizeof(T);
        return v;
    }
    template <class T>
    bool getArray(std::vector<T>& out, std::uint64_t n) {
        if (!ok || n > left / sizeof(T)) return ok = false;
        out.resize((std::size_t)n);
        if (n) std::memcpy(out.data(), p, (std::size_t)n * sizeof(T));
        p += n * sizeof(T);
        left -= n * sizeof(T);
        return true;
    }
};

std::uint64_t fnv1a(const unsigned char* p, std::size_t n) {
    std::uint64_t h = 0xcbf29ce484222325ull;
    for (std::size_t i = 0; i < n; ++i) {
        h ^= p[i];
        h *= 0x100000001b3ull;
    }
    return h;
}

}  // namespace

struct symgb_plan_file {
    symgb_plan_desc desc{};
    std::vector<symgb_kernel_desc> kernels;
    std::vector<std::vector<symgb_node>> nodes;
    std::vector<std::vector<std::int32_t>> access;
    std::vector<std::uint64_t> argStart, argLength, outStart, outLength;
    std::vector<std::uint32_t> indexData, outIndexData;
    std::vector<double> constData;
};

extern "C" {

const char* symgb_plan_last_error(void) { return g_planError.c_str(); }

int symgb_plan_save(const char* path, const symgb_plan_desc* d, const uint32_t* index_data,
                    const uint32_t* out_index_data, const double* const_data) {
    if (!path || !d) return planFail("null argument");
    if ((d->num_kernels && !d->kernels) || (d->num_args && (!d->arg_start || !d->arg_length)) ||
        (d->num_outputs && (!d->output_start || !d->output_length)) || (d->num_indices && !index_data) ||
        (d->num_output_values && !out_index_data) || (d->num_constants && !const_data))
        return planFail("plan description has null arrays");
    Writer w;
    w.putArray(kMagic, 8);
    w.put(kVersion);
    w.put(kByteOrder);
    w.put(d->num_kernels);
    w.put(d->num_args);
    w.put(d->num_outputs);
    w.put(d->threads_per_block);
    w.put(d->num_total_memory);
    w.put(d->num_indices);
    w.put(d->num_output_values);
    w.put(d->num_constants);
    w.putArray(d->arg_start, d->num_args);
    w.putArray(d->arg_length, d->num_args);
    w.putArray(d->output_start, d->num_outputs);
    w.putArray(d->output_length, d->num_outputs);
    for (std::uint32_t k = 0; k < d->num_kernels; ++k) {
        const symgb_kernel_desc& K = d->kernels[k];
        if ((K.num_nodes && !K.nodes) || (K.num_access && !K.access)) return planFail("kernel has null arrays");
        w.put(K.num_instances);
        w.put(K.output_offset);
        w.put(K.index_offset);
        w.put(K.constants_offset);
        w.put(K.num_output_rows);
        w.put(K.num_index_rows);
        w.put(K.num_constant_rows);
        w.put(K.level);
        w.put(K.num_nodes);
        for (std::uint32_t j = 0; j < K.num_nodes; ++j) {
            w.put(K.nodes[j].op);
            w.put(K.nodes[j].nchild);
            w.put(K.nodes[j].a);
            w.put(K.nodes[j].b);
            w.put(K.nodes[j].value);
        }
        w.put(K.num_access);
        w.putArray(K.access, 2 * (std::size_t)K.num_access);
    }
    w.putArray(index_data, d->num_indices);
    w.putArray(out_index_data, d->num_output_values);
    w.putArray(const_data, d->num_constants);
    const std::uint64_t sum = fnv1a(w.buf.data(), w.buf.size());
    w.put(sum);
    std::FILE* f = std::fopen(path, "wb");
    if (!f) return planFail(std::string("cannot open ") + path + " for writing");
    const bool ok = std::fwrite(w.buf.data(), 1, w.buf.size(), f) == w.buf.size();
    if (std::fclose(f) != 0 || !ok) return planFail(std::string("cannot write ") + path);
    return SYMGB_OK;
}

int symgb_plan_load(const char* path, symgb_plan_file_t* out) {
    if (!path || !out) return planFail("null argument");
    *out = nullptr;
    std::FILE* f = std::fopen(path, "rb");
    if (!f) return planFail(std::string("cannot open ") + path);
    std::vector<unsigned char> buf;
    unsigned char chunk[1 << 16];
    std::size_t got;
    while ((got = std::fread(chunk, 1, sizeof(chunk), f)) > 0) buf.insert(buf.end(), chunk, chunk + got);
    std::fclose(f);
    if (buf.size() < 8 + 8 + 8 || std::memcmp(buf.data(), kMagic, 8) != 0) return planFail("not a plan file");
    std::uint64_t sum;
    std::memcpy(&sum, buf.data() + buf.size() - 8, 8);
    if (fnv1a(buf.data(), buf.size() - 8) != sum) return planFail("plan file checksum mismatch");
    Reader r{buf.data() + 8, buf.size() - 8 - 8};
    if (r.get<std::uint32_t>() != kVersion) return planFail("unsupported plan file version");
    if (r.get<std::uint32_t>() != kByteOrder) return planFail("plan file byte order differs");
    auto pf = std::make_unique<symgb_plan_file>();
    symgb_plan_desc& d = pf->desc;
    d.num_kernels = r.get<std::uint32_t>();
    d.num_args = r.get<std::uint32_t>();
    d.num_outputs = r.get<std::uint32_t>();
    d.threads_per_block = r.get<std::uint32_t>();
    d.num_total_memory = r.get<std::uint64_t>();
    d.num_indices = r.get<std::uint64_t>();
    d.num_output_values = r.get<std::uint64_t>();
    d.num_constants = r.get<std::uint64_t>();
    r.getArray(pf->argStart, d.num_args);
    r.getArray(pf->argLength, d.num_args);
    r.getArray(pf->outStart, d.num_outputs);
    r.getArray(pf->outLength, d.num_outputs);
    if (!r.ok || d.num_kernels > r.left) return planFail("truncated plan file");
    pf->kernels.resize(d.num_kernels);
    pf->nodes.resize(d.num_kernels);
    pf->access.resize(d.num_kernels);
    for (std::uint32_t k = 0; k < d.num_kernels && r.ok; ++k) {
        symgb_kernel_desc& K = pf->kernels[k];
        K.num_instances = r.get<std::uint64_t>();
        K.output_offset = r.get<std::uint64_t>();
        K.index_offset = r.get<std::uint64_t>();
        K.constants_offset = r.get<std::uint64_t>();
        K.num_output_rows = r.get<std::uint32_t>();
        K.num_index_rows = r.get<std::uint32_t>();
        K.num_constant_rows = r.get<std::uint32_t>();
        K.level = r.get<std::int32_t>();
        K.num_nodes = r.get<std::uint32_t>();
        if (!r.ok || K.num_nodes > r.left / 24) return planFail("truncated plan file");
        pf->nodes[k].resize(K.num_nodes);
        for (auto& nd : pf->nodes[k]) {
            nd.op = r.get<std::int32_t>();
            nd.nchild = r.get<std::int32_t>();
            nd.a = r.get<std::int32_t>();
            nd.b = r.get<std::int32_t>();
            nd.value = r.get<double>();
        }
        K.num_access = r.get<std::uint32_t>();
        r.getArray(pf->access[k], 2 * (std::uint64_t)K.num_access);
        K.nodes = pf->nodes[k].data();
        K.access = pf->access[k].data();
    }
    r.getArray(pf->indexData, d.num_indices);
    r.getArray(pf->outIndexData, d.num_output_values);
    r.getArray(pf->constData, d.num_constants);
    if (!r.ok || r.left != 0) return planFail("truncated or oversized plan file");
    d.kernels = pf->kernels.data();
    d.arg_start = pf->argStart.data();
    d.arg_length = pf->argLength.data();
    d.output_start = pf->outStart.data();
    d.output_length = pf->outLength.data();
    *out = pf.release();
    return SYMGB_OK;
}

const symgb_plan_desc* symgb_plan_file_desc(symgb_plan_file_t f) { return f ? &f->desc : nullptr; }
const uint32_t* symgb_plan_file_index_data(symgb_plan_file_t f) { return f ? f->indexData.data() : nullptr; }
const uint32_t* symgb_plan_file_out_index_data(symgb_plan_file_t f) { return f ? f->outIndexData.data() : nullptr; }
const double* symgb_plan_file_const_data(symgb_plan_file_t f) { return f ? f->constData.data() : nullptr; }
void symgb_plan_file_free(symgb_plan_file_t f) { delete f; }

}  // extern "C"
