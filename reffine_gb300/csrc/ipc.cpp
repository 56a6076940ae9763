// Arrow IPC file ingest: the first record batch of an Arrow IPC file as Arrow C data
// (rf_ipc_read), or straight into a device table (rf_table_load_ipc).
//
// The reference loads its benchmark tables with load_arrow_file (src/utils/utils.cpp:11-34):
// Arrow C++'s RecordBatchFileReader reads record batch 0, ExportRecordBatch turns it into the
// C data of an ArrowTable2.  Arrow C++ is not part of this backend, so the file is parsed here:
// the IPC file format (magic, footer, encapsulated messages) and the FlatBuffers tables of the
// Arrow format (Footer, Schema, Field, Int, FloatingPoint, Message, RecordBatch) as published in
// the Arrow project's format specification.  Every offset read from the file is checked against
// the file's size; anything outside the supported subset - compressed bodies, dictionaries,
// types other than integers, floats and run-end encoded columns of them - is refused with a
// message, never read.
#include <fcntl.h>
#include <sys/mman.h>
#include <sys/stat.h>
#include <unistd.h>

#include <cerrno>
#include <cstdlib>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <deque>
#include <memory>
#include <string>
#include <vector>

#include "objects.h"
#include "reffine_gb300/arrow_c.h"
#include "rf_gpu.h"
#include "runtime.h"

namespace {

struct IpcError {
    std::string msg;
};

// a FlatBuffers view over the file, every read bounds-checked
struct Buf {
    const uint8_t* p;
    size_t n;

    void need(size_t off, size_t len) const
    {
        if (off > n || len > n - off) throw IpcError{"offset outside the file (corrupt or truncated)"};
    }
    template <class T>
    T at(size_t off) const
    {
        need(off, sizeof(T));
        T v;
        std::memcpy(&v, p + off, sizeof(T));
        return v;
    }
};

// a FlatBuffers table at `pos`: its vtable gives each field's offset inside the table
struct Table {
    const Buf* b;
    size_t pos = 0, vt = 0, vt_size = 0;

    Table(const Buf* buf, size_t at) : b(buf), pos(at)
    {
        const int32_t soff = b->at<int32_t>(pos);
        const long long v = (long long)pos - soff;
        if (v < 0) throw IpcError{"bad vtable offset"};
        vt = (size_t)v;
        vt_size = b->at<uint16_t>(vt);
        if (vt_size < 4) throw IpcError{"bad vtable"};
        b->need(vt, vt_size);
    }
    // position of field i, 0 when absent
    size_t field(int i) const
    {
        const size_t e = 4 + 2 * (size_t)i;
        if (e + 2 > vt_size) return 0;
        const uint16_t off = b->at<uint16_t>(vt + e);
        return off ? pos + off : 0;
    }
    template <class T>
    T scalar(int i, T dflt) const
    {
        const size_t f = field(i);
        return f ? b->at<T>(f) : dflt;
    }
    // target of an offset field (table, vector or string), 0 when absent
    size_t ref(int i) const
    {
        const size_t f = field(i);
        if (!f) return 0;
        return f + b->at<uint32_t>(f);
    }
};

// a FlatBuffers vector at `v`: [u32 length][elements]
struct Vec {
    size_t at = 0, len = 0;
    Vec() = default;
    Vec(const Buf* b, size_t v, size_t elem)
    {
        if (!v) return;
        len = b->at<uint32_t>(v);
        at = v + 4;
        if (elem && len > (b->n / elem)) throw IpcError{"vector longer than the file"};
        b->need(at, len * elem);
    }
};

std::string str(const Buf* b, size_t s)
{
    if (!s) return "";
    const uint32_t n = b->at<uint32_t>(s);
    b->need(s + 4, n);
    return std::string((const char*)b->p + s + 4, n);
}

// Type union members of the Arrow schema (Schema.fbs)
enum : uint8_t { kInt = 2, kFloatingPoint = 3, kRunEndEncoded = 22 };

// everything the exported C data points into; freed when both top-level objects are released
struct Holder {
    std::vector<uint8_t> file;
    std::deque<ArrowSchema> schemas;
    std::deque<ArrowArray> arrays;
    std::deque<std::vector<const void*>> buffers;
    std::deque<std::vector<ArrowSchema*>> schema_kids;
    std::deque<std::vector<ArrowArray*>> array_kids;
    std::deque<std::string> strings;
    int refs = 2;
};

void release_child_schema(ArrowSchema* s) { s->release = nullptr; }
void release_child_array(ArrowArray* a) { a->release = nullptr; }
void drop(Holder* h)
{
    if (--h->refs == 0) delete h;
}
void release_top_schema(ArrowSchema* s)
{
    Holder* h = (Holder*)s->private_data;
    s->release = nullptr;
    drop(h);
}
void release_top_array(ArrowArray* a)
{
    Holder* h = (Holder*)a->private_data;
    a->release = nullptr;
    drop(h);
}

struct Reader {
    Buf b;
    Holder* h;
    size_t body = 0, body_len = 0;
    Vec nodes, bufs;
    size_t next_node = 0, next_buf = 0;

    const char* keep(const std::string& s)
    {
        h->strings.push_back(s);
        return h->strings.back().c_str();
    }

    void node(long long& length, long long& nulls)
    {
        if (next_node >= nodes.len) throw IpcError{"record batch has fewer field nodes than the schema needs"};
        const size_t at = nodes.at + 16 * next_node++;
        length = b.at<int64_t>(at);
        nulls = b.at<int64_t>(at + 8);
        if (length < 0 || nulls < 0 || nulls > length) throw IpcError{"bad field node"};
    }

    // the next buffer of the batch: at least `min_len` bytes, and `read_len` bytes of the body
    // from its start (a validity bitmap is read as whole 16-bit words, past its stated length
    // into the 8-byte padding the format requires)
    const void* buffer(size_t min_len, size_t read_len)
    {
        if (next_buf >= bufs.len) throw IpcError{"record batch has fewer buffers than the schema needs"};
        const size_t at = bufs.at + 16 * next_buf++;
        const int64_t off = b.at<int64_t>(at), len = b.at<int64_t>(at + 8);
        if (off < 0 || len < 0 || (uint64_t)off > body_len || (uint64_t)len > body_len - (uint64_t)off)
            throw IpcError{"buffer outside the record batch body"};
        if (len == 0) return nullptr;
        if ((size_t)len < min_len || read_len > body_len - (size_t)off) throw IpcError{"buffer shorter than its column"};
        return b.p + body + (size_t)off;
    }

    // one field (and its children) of the schema, with the matching nodes and buffers
    void field(size_t fpos, ArrowSchema* s, ArrowArray* a)
    {
        Table f(&b, fpos);
        if (f.ref(4)) throw IpcError{"dictionary-encoded columns are not supported"};
        const std::string name = str(&b, f.ref(0));
        const uint8_t tt = f.scalar<uint8_t>(2, 0);
        const size_t tpos = f.ref(3);
        std::memset(s, 0, sizeof *s);
        std::memset(a, 0, sizeof *a);
        s->name = keep(name);
        s->flags = f.scalar<uint8_t>(1, 0) ? ARROW_FLAG_NULLABLE : 0;
        s->release = release_child_schema;
        a->release = release_child_array;
        long long length, nulls;
        node(length, nulls);
        a->length = length;
        a->null_count = nulls;
        if (tt == kInt || tt == kFloatingPoint) {
            if (!tpos) throw IpcError{"field without its type"};
            Table t(&b, tpos);
            size_t width;
            if (tt == kInt) {
                const int32_t bits = t.scalar<int32_t>(0, 0);
                const bool sgn = t.scalar<uint8_t>(1, 0) != 0;
                static const char* fs[] = {"c", "s", "i", "l"}, *fu[] = {"C", "S", "I", "L"};
                const int k = bits == 8 ? 0 : bits == 16 ? 1 : bits == 32 ? 2 : bits == 64 ? 3 : -1;
                if (k < 0) throw IpcError{"integer width " + std::to_string(bits) + " in column " + name};
                s->format = sgn ? fs[k] : fu[k];
                width = (size_t)bits / 8;
            } else {
                const int16_t prec = t.scalar<int16_t>(0, 0);
                if (prec == 1) s->format = "f", width = 4;
                else if (prec == 2) s->format = "g", width = 8;
                else throw IpcError{"half-precision column " + name + " is not supported"};
            }
            const void* valid = buffer((size_t)(length + 7) / 8, (size_t)(length + 15) / 16 * 2);
            const void* values = buffer((size_t)length * width, (size_t)length * width);
            h->buffers.push_back({valid, values});
            a->n_buffers = 2;
            a->buffers = h->buffers.back().data();
            return;
        }
        if (tt == kRunEndEncoded) {
            // no buffers of its own; children: run ends (int32), values
            Vec kids(&b, f.ref(5), 4);
            if (kids.len != 2) throw IpcError{"run-end encoded column " + name + " without its two children"};
            s->format = "+r";
            // deque elements keep their addresses as the deque grows at its end
            ArrowSchema* cs[2];
            ArrowArray* ca[2];
            for (int c = 0; c < 2; c++) {
                h->schemas.emplace_back();
                h->arrays.emplace_back();
                cs[c] = &h->schemas.back();
                ca[c] = &h->arrays.back();
            }
            for (int c = 0; c < 2; c++) {
                const size_t e = kids.at + 4 * (size_t)c;
                field(e + b.at<uint32_t>(e), cs[c], ca[c]);
            }
            if (std::string(cs[0]->format) != "i") throw IpcError{"run ends of column " + name + " must be int32"};
            h->schema_kids.push_back({cs[0], cs[1]});
            h->array_kids.push_back({ca[0], ca[1]});
            s->n_children = 2;
            s->children = h->schema_kids.back().data();
            a->n_children = 2;
            a->children = h->array_kids.back().data();
            h->buffers.push_back({nullptr});
            a->n_buffers = 0;
            a->buffers = h->buffers.back().data();
            return;
        }
        throw IpcError{"column " + name + ": type " + std::to_string(tt) +
                       " is not supported (integers, floats and run-end encoded columns are)"};
    }
};

// Parses record batch 0 of the IPC file image `b` into Arrow C data whose buffers point into
// the image; `h` keeps the exported structs (and, for rf_ipc_read, the image itself).
int parse_file(const Buf& b, Holder* h, ArrowSchema* schema, ArrowArray* array, std::string& err)
{
    std::memset(schema, 0, sizeof *schema);
    std::memset(array, 0, sizeof *array);
    try {
        Reader r{b, h, 0, 0, Vec(), Vec(), 0, 0};
        // file: "ARROW1" 2 bytes of padding ... footer, int32 footer size, "ARROW1"
        if (b.n < 18 || std::memcmp(b.p, "ARROW1", 6) != 0 || std::memcmp(b.p + b.n - 6, "ARROW1", 6) != 0)
            throw IpcError{"not an Arrow IPC file (magic)"};
        const int32_t flen = b.at<int32_t>(b.n - 10);
        if (flen <= 0 || (size_t)flen > b.n - 18) throw IpcError{"bad footer length"};
        const size_t fstart = b.n - 10 - (size_t)flen;
        Table footer(&b, fstart + b.at<uint32_t>(fstart));
        const size_t spos = footer.ref(1);
        if (!spos) throw IpcError{"footer without a schema"};
        Table sch(&b, spos);
        if (sch.scalar<int16_t>(0, 0) != 0) throw IpcError{"big-endian files are not supported"};
        Vec fields(&b, sch.ref(1), 4);
        Vec batches(&b, footer.ref(3), 24);
        if (batches.len == 0) throw IpcError{"the file has no record batch"};
        // record batch 0: block {offset, metadata length, body length}
        const int64_t boff = b.at<int64_t>(batches.at), blen = b.at<int64_t>(batches.at + 16);
        const int32_t mlen = b.at<int32_t>(batches.at + 8);
        if (boff < 8 || mlen <= 0 || blen < 0) throw IpcError{"bad record batch block"};
        b.need((size_t)boff, (size_t)mlen);
        b.need((size_t)boff + (size_t)mlen, (size_t)blen);
        // encapsulated message: [0xFFFFFFFF][int32 length] flatbuffer, or the older [int32 length]
        size_t mpos = (size_t)boff;
        if (b.at<uint32_t>(mpos) == 0xFFFFFFFFu) mpos += 4;
        mpos += 4;
        Table msg(&b, mpos + b.at<uint32_t>(mpos));
        if (msg.scalar<uint8_t>(1, 0) != 3) throw IpcError{"record batch block does not hold a record batch"};
        const size_t rpos = msg.ref(2);
        if (!rpos) throw IpcError{"message without its record batch"};
        Table rb(&b, rpos);
        if (rb.ref(3)) throw IpcError{"compressed record batches are not supported"};
        const int64_t rows = rb.scalar<int64_t>(0, 0);
        r.nodes = Vec(&b, rb.ref(1), 16);
        r.bufs = Vec(&b, rb.ref(2), 16);
        r.body = (size_t)boff + (size_t)mlen;
        r.body_len = (size_t)blen;
        // the top-level struct of columns (ArrowTable2's layout: "+s" with one child per column)
        const size_t n = fields.len;
        for (size_t i = 0; i < n; i++) {
            h->schemas.emplace_back();
            h->arrays.emplace_back();
        }
        std::vector<ArrowSchema*> ks;
        std::vector<ArrowArray*> ka;
        for (size_t i = 0; i < n; i++) {
            ks.push_back(&h->schemas[i]);
            ka.push_back(&h->arrays[i]);
        }
        for (size_t i = 0; i < n; i++) {
            const size_t e = fields.at + 4 * i;
            r.field(e + b.at<uint32_t>(e), ks[i], ka[i]);
            if (ka[i]->length != rows) throw IpcError{"column length differs from the record batch's"};
        }
        h->schema_kids.push_back(ks);
        h->array_kids.push_back(ka);
        h->buffers.push_back({nullptr});
        schema->format = "+s";
        schema->name = "";
        schema->n_children = (int64_t)n;
        schema->children = h->schema_kids.back().data();
        schema->release = release_top_schema;
        schema->private_data = h;
        array->length = rows;
        array->n_buffers = 1;
        array->buffers = h->buffers.back().data();
        array->n_children = (int64_t)n;
        array->children = h->array_kids.back().data();
        array->release = release_top_array;
        array->private_data = h;
        return RF_OK;
    } catch (const IpcError& e) {
        err = e.msg;
        std::memset(schema, 0, sizeof *schema);
        std::memset(array, 0, sizeof *array);
        return e.msg.find("not supported") != std::string::npos ? RF_ERR_UNSUPPORTED : RF_ERR_INVALID;
    }
}

// the file's bytes [off, off + n) into dst, whole (pread returns short counts near page-cache
// boundaries and on signals)
bool pread_all(int fd, void* dst, size_t n, size_t off)
{
    char* d = (char*)dst;
    while (n) {
        const ssize_t got = ::pread(fd, d, n, (off_t)off);
        if (got < 0 && errno == EINTR) continue;
        if (got <= 0) return false;
        d += got, off += (size_t)got, n -= (size_t)got;
    }
    return true;
}

}  // namespace

extern "C" int rf_ipc_read(const char* path, ArrowSchema* schema, ArrowArray* array, char* err, size_t err_len)
{
    auto put = [&](const std::string& m) {
        if (err && err_len) {
            size_t n = std::min(err_len - 1, m.size());
            std::memcpy(err, m.data(), n);
            err[n] = 0;
        }
    };
    if (!path || !schema || !array) {
        put("null argument");
        return RF_ERR_INVALID;
    }
    std::memset(schema, 0, sizeof *schema);
    std::memset(array, 0, sizeof *array);
    std::unique_ptr<Holder> h(new Holder);
    {
        FILE* f = std::fopen(path, "rb");
        if (!f) {
            put(std::string("cannot open ") + path);
            return RF_ERR_INVALID;
        }
        std::fseek(f, 0, SEEK_END);
        long sz = std::ftell(f);
        std::fseek(f, 0, SEEK_SET);
        if (sz < 0) sz = 0;
        h->file.resize((size_t)sz);
        size_t got = sz ? std::fread(h->file.data(), 1, (size_t)sz, f) : 0;
        std::fclose(f);
        if (got != (size_t)sz) {
            put(std::string("cannot read ") + path);
            return RF_ERR_INVALID;
        }
    }
    std::string msg;
    const int rc = parse_file(Buf{h->file.data(), h->file.size()}, h.get(), schema, array, msg);
    if (rc) {
        put(msg);
        return rc;
    }
    h.release();  // owned by the two exported objects now
    return RF_OK;
}

// The file is mapped and parsed in place (the parser touches only the footer and the message
// metadata).  Where the GPU reads pageable memory through the host page tables (Grace hosts) the
// mapping is populated up front and the column buffers are copied straight out of it by DMA: one
// pass over the page cache, no host copy.  Elsewhere host threads pread slices of the column
// buffers into the pinned staging ring while the previous slices' DMA runs (staged_h2d).
// RF_IPC_LOAD=staged selects the second path on any host.
extern "C" int rf_table_load_ipc(rf_ctx* ctx, const char* path, int64_t dim, void* stream, rf_table** out)
{
    if (!ctx || !out || !path) return ctx ? rfrt::fail(ctx, RF_ERR_INVALID, "null argument") : RF_ERR_INVALID;
    *out = nullptr;
    cudaSetDevice(ctx->device);
    cudaStream_t s = stream ? (cudaStream_t)stream : ctx->stream;
    const char* mode = std::getenv("RF_IPC_LOAD");
    const bool direct = ctx->pageable_direct && !(mode && std::strcmp(mode, "staged") == 0);
    const int fd = ::open(path, O_RDONLY | O_CLOEXEC);
    if (fd < 0) return rfrt::fail(ctx, RF_ERR_INVALID, "cannot open %s", path);
    struct stat st;
    if (::fstat(fd, &st) != 0 || st.st_size < 18) {
        ::close(fd);
        return rfrt::fail(ctx, RF_ERR_INVALID, "%s: not an Arrow IPC file (too short)", path);
    }
    const size_t size = (size_t)st.st_size;
    void* map = ::mmap(nullptr, size, PROT_READ, MAP_PRIVATE | (direct ? MAP_POPULATE : 0), fd, 0);
    if (map == MAP_FAILED) {
        ::close(fd);
        return rfrt::fail(ctx, RF_ERR_INVALID, "cannot map %s", path);
    }
    if (!direct) ::posix_fadvise(fd, 0, 0, POSIX_FADV_SEQUENTIAL);
    const uint8_t* base = (const uint8_t*)map;
    ArrowSchema sc;
    ArrowArray ar;
    std::string msg;
    Holder* h = new Holder;
    int rc = parse_file(Buf{base, size}, h, &sc, &ar, msg);
    if (rc) {
        delete h;
        rc = rfrt::fail(ctx, rc, "%s", msg.c_str());
    } else {
        if (direct) {
            rc = rfrt::upload(ctx, &sc, &ar, dim, nullptr, 0, s, out, nullptr);
            // the mapping is unmapped next: the copies out of it must have landed
            const cudaError_t e = cudaStreamSynchronize(s);
            if (!rc && e != cudaSuccess) rc = rfrt::fail(ctx, RF_ERR_CUDA, "copy from %s: %s", path, cudaGetErrorString(e));
        } else {
            std::vector<rfrt::HostCopy> copies;
            rc = rfrt::upload(ctx, &sc, &ar, dim, nullptr, 0, s, out, nullptr, &copies);
            if (!rc)
                rc = rfrt::staged_h2d(ctx, copies, [&](void* dst, const void* src, size_t n) {
                    return pread_all(fd, dst, n, (size_t)((const uint8_t*)src - base));
                }, s);
        }
        if (rc && *out) {
            rf_table_free(*out);
            *out = nullptr;
        }
        ar.release(&ar);
        sc.release(&sc);
    }
    ::munmap(map, size);
    ::close(fd);
    return rc;
}
