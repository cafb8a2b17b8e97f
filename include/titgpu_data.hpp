/*
 * titgpu_data.hpp - the .ttdb particle storage of TitSolver
 * (source/tit/data/storage.hpp, storage.cpp:30-67), written by the C++ host
 * mirror so that existing readers open GPU results.
 *
 * Format (kept identical to the reference, since readers depend on it):
 *   - an SQLite database with tables Settings(id = 0, max_series),
 *     DataSeries(id, name), DataFrames(id, series_id, time) and
 *     DataArrays(id, frame_id, name, type, size, data), foreign keys with
 *     ON DELETE CASCADE, journal_mode WAL;
 *   - DataArrays.type = (kind + 1) | rank << 8 | dim << 16 with kind ids
 *     int8 0, uint8 1, int16 2, uint16 3, int32 4, uint32 5, int64 6,
 *     uint64 7, float32 8, float64 9 and rank scalar 0, vector 1, matrix 2
 *     (source/tit/data/type.hpp:179-189); size = number of elements;
 *   - DataArrays.data = the elements' bytes as one zstd frame (RFC 8878).
 *
 * SQLite is reached through the system's libsqlite3.so.0, opened at run
 * time (no headers or link-time dependency).  The zstd frames are written by
 * this header with raw (stored) blocks, which every zstd decoder reads; the
 * payload is not compressed.
 *
 * Writes of a frame can run on a background thread (Storage::write_frame_async)
 * so that the device keeps stepping while the host writes the previous
 * snapshot; every other call waits for the pending write first.
 */
#ifndef TITGPU_DATA_HPP
#define TITGPU_DATA_HPP

#include <dlfcn.h>

#include <cstddef>
#include <cstdint>
#include <cstring>
#include <exception>
#include <filesystem>
#include <future>
#include <memory>
#include <span>
#include <string>
#include <string_view>
#include <type_traits>
#include <utility>
#include <vector>

#include "titgpu.hpp"

namespace tit::data {

// ---- zstd frame with raw blocks (RFC 8878, sections 3.1.1 and 3.1.1.2) ------
namespace zstd_raw {

inline void put_le(std::vector<std::byte>& out, std::uint64_t v, int bytes) {
  for (int i = 0; i < bytes; ++i) {
    out.push_back(static_cast<std::byte>((v >> (8 * i)) & 0xffu));
  }
}

/// One zstd frame holding `data`: magic 0xFD2FB528, a single-segment frame
/// header with an 8-byte content size, then raw blocks of at most 128 KiB
/// (the block size limit), the last one flagged.
inline auto encode(std::span<const std::byte> data) -> std::vector<std::byte> {
  constexpr std::size_t max_block = std::size_t{128} * 1024;
  std::vector<std::byte> out;
  out.reserve(data.size() + 13 + 3 * (data.size() / max_block + 1));
  put_le(out, 0xFD2FB528u, 4);
  // Frame_Header_Descriptor: FCS_Field_Size = 3 (8 bytes), Single_Segment.
  out.push_back(static_cast<std::byte>(0xE0));
  put_le(out, data.size(), 8);
  std::size_t pos = 0;
  do {
    const std::size_t len = std::min(max_block, data.size() - pos);
    const bool last = pos + len == data.size();
    // Block_Header: Last_Block (bit 0), Block_Type Raw = 0 (bits 1-2),
    // Block_Size (bits 3-23).
    put_le(out, (static_cast<std::uint64_t>(len) << 3) | (last ? 1u : 0u), 3);
    out.insert(out.end(), data.begin() + static_cast<std::ptrdiff_t>(pos),
               data.begin() + static_cast<std::ptrdiff_t>(pos + len));
    pos += len;
  } while (pos < data.size());
  return out;
}

} // namespace zstd_raw

// ---- data types (source/tit/data/type.hpp) ---------------------------------
enum class KindID : std::uint8_t {
  int8, uint8, int16, uint16, int32, uint32, int64, uint64, float32, float64
};
enum class Rank : std::uint8_t { scalar, vector, matrix };

template<class T>
constexpr auto kind_of() -> KindID {
  if constexpr (std::is_same_v<T, std::int8_t>) return KindID::int8;
  else if constexpr (std::is_same_v<T, std::uint8_t>) return KindID::uint8;
  else if constexpr (std::is_same_v<T, std::int16_t>) return KindID::int16;
  else if constexpr (std::is_same_v<T, std::uint16_t>) return KindID::uint16;
  else if constexpr (std::is_same_v<T, std::int32_t>) return KindID::int32;
  else if constexpr (std::is_same_v<T, std::uint32_t>) return KindID::uint32;
  else if constexpr (std::is_same_v<T, std::int64_t>) return KindID::int64;
  else if constexpr (std::is_same_v<T, std::uint64_t>) return KindID::uint64;
  else if constexpr (std::is_same_v<T, float>) return KindID::float32;
  else {
    static_assert(std::is_same_v<T, double>, "unsupported element kind");
    return KindID::float64;
  }
}

constexpr auto type_id(KindID kind, Rank rank, std::uint8_t dim)
    -> std::uint32_t {
  return (static_cast<std::uint32_t>(kind) + 1u) |
         static_cast<std::uint32_t>(rank) << 8 |
         static_cast<std::uint32_t>(dim) << 16;
}

template<class T>
struct element_type {
  static constexpr std::uint32_t id = type_id(kind_of<T>(), Rank::scalar, 1);
};
template<class Real, std::size_t Dim>
struct element_type<Vec<Real, Dim>> {
  static constexpr std::uint32_t id =
      type_id(kind_of<Real>(), Rank::vector, static_cast<std::uint8_t>(Dim));
};

/// One named array of a frame: its type id, element count and bytes.
struct ArrayBlob {
  std::string name;
  std::uint32_t type = 0;
  std::int64_t size = 0;
  std::vector<std::byte> bytes;

  template<class T>
  static auto of(std::string name, std::span<const T> values) -> ArrayBlob {
    static_assert(std::is_trivially_copyable_v<T>);
    ArrayBlob a;
    a.name = std::move(name);
    a.type = element_type<T>::id;
    a.size = static_cast<std::int64_t>(values.size());
    const auto* p = reinterpret_cast<const std::byte*>(values.data());
    a.bytes.assign(p, p + values.size_bytes());
    return a;
  }
};

// ---- SQLite through the C API of libsqlite3.so.0 ---------------------------
namespace sqlite {

struct Api {
  using Open = int (*)(const char*, void**, int, const char*);
  using Close = int (*)(void*);
  using Exec = int (*)(void*, const char*, void*, void*, char**);
  using Prepare = int (*)(void*, const char*, int, void**, const char**);
  using BindI64 = int (*)(void*, int, std::int64_t);
  using BindF64 = int (*)(void*, int, double);
  using BindText = int (*)(void*, int, const char*, int, void (*)(void*));
  using BindBlob64 = int (*)(void*, int, const void*, std::uint64_t,
                             void (*)(void*));
  using Step = int (*)(void*);
  using Finalize = int (*)(void*);
  using ColI64 = std::int64_t (*)(void*, int);
  using LastRowId = std::int64_t (*)(void*);
  using ErrMsg = const char* (*)(void*);
  using Free = void (*)(void*);

  Open open = nullptr;
  Close close = nullptr;
  Exec exec = nullptr;
  Prepare prepare = nullptr;
  BindI64 bind_int64 = nullptr;
  BindF64 bind_double = nullptr;
  BindText bind_text = nullptr;
  BindBlob64 bind_blob64 = nullptr;
  Step step = nullptr;
  Finalize finalize = nullptr;
  ColI64 column_int64 = nullptr;
  LastRowId last_insert_rowid = nullptr;
  ErrMsg errmsg = nullptr;
  Free free = nullptr;

  static constexpr int ok = 0;
  static constexpr int row = 100;
  static constexpr int done = 101;
  static constexpr int open_readwrite = 0x2;
  static constexpr int open_create = 0x4;

  static auto get() -> const Api& {
    static const Api api = load();
    return api;
  }

private:
  static auto load() -> Api {
    void* lib = dlopen("libsqlite3.so.0", RTLD_NOW | RTLD_LOCAL);
    if (lib == nullptr) lib = dlopen("libsqlite3.so", RTLD_NOW | RTLD_LOCAL);
    if (lib == nullptr) {
      throw Exception{"Storage: libsqlite3.so.0 is not available"};
    }
    Api a;
    const auto sym = [lib](auto& fn, const char* name) {
      fn = reinterpret_cast<std::remove_reference_t<decltype(fn)>>(
          dlsym(lib, name));
      if (fn == nullptr) {
        throw Exception{std::string{"Storage: libsqlite3 lacks "} + name};
      }
    };
    sym(a.open, "sqlite3_open_v2");
    sym(a.close, "sqlite3_close");
    sym(a.exec, "sqlite3_exec");
    sym(a.prepare, "sqlite3_prepare_v2");
    sym(a.bind_int64, "sqlite3_bind_int64");
    sym(a.bind_double, "sqlite3_bind_double");
    sym(a.bind_text, "sqlite3_bind_text");
    sym(a.bind_blob64, "sqlite3_bind_blob64");
    sym(a.step, "sqlite3_step");
    sym(a.finalize, "sqlite3_finalize");
    sym(a.column_int64, "sqlite3_column_int64");
    sym(a.last_insert_rowid, "sqlite3_last_insert_rowid");
    sym(a.errmsg, "sqlite3_errmsg");
    sym(a.free, "sqlite3_free");
    return a;
  }
};

// SQLITE_TRANSIENT: SQLite copies bound text and blobs.
inline auto transient() -> void (*)(void*) {
  return reinterpret_cast<void (*)(void*)>(static_cast<std::intptr_t>(-1));
}

class Database {
public:
  explicit Database(const std::filesystem::path& path) : api_{&Api::get()} {
    void* db = nullptr;
    const int st = api_->open(path.c_str(), &db,
                              Api::open_readwrite | Api::open_create, nullptr);
    if (st != Api::ok) {
      std::string msg = "Storage: cannot open '" + path.string() + "'";
      if (db != nullptr) {
        msg += std::string{": "} + api_->errmsg(db);
        api_->close(db);
      }
      throw Exception{msg};
    }
    db_ = db;
  }
  Database(const Database&) = delete;
  auto operator=(const Database&) -> Database& = delete;
  ~Database() {
    if (db_ != nullptr) api_->close(db_);
  }

  void execute(const char* sql) {
    char* err = nullptr;
    if (api_->exec(db_, sql, nullptr, nullptr, &err) != Api::ok) {
      std::string msg = std::string{"Storage: SQL failed: "} +
                        (err != nullptr ? err : api_->errmsg(db_));
      if (err != nullptr) api_->free(err);
      throw Exception{msg};
    }
  }

  /// Run one statement; `bind(stmt)` binds its parameters.  Returns the
  /// first column of the first row (0 when there is none).
  template<class Bind>
  auto run(const char* sql, Bind&& bind) -> std::int64_t {
    void* stmt = nullptr;
    if (api_->prepare(db_, sql, -1, &stmt, nullptr) != Api::ok) {
      throw Exception{std::string{"Storage: prepare failed: "} +
                      api_->errmsg(db_)};
    }
    bind(*api_, stmt);
    std::int64_t first = 0;
    const int st = api_->step(stmt);
    if (st == Api::row) first = api_->column_int64(stmt, 0);
    const int fin = api_->finalize(stmt);
    if ((st != Api::row && st != Api::done) || fin != Api::ok) {
      throw Exception{std::string{"Storage: statement failed: "} +
                      api_->errmsg(db_)};
    }
    return first;
  }
  auto run(const char* sql) -> std::int64_t {
    return run(sql, [](const Api&, void*) {});
  }
  auto last_insert_rowid() const -> std::int64_t {
    return api_->last_insert_rowid(db_);
  }

private:
  const Api* api_;
  void* db_ = nullptr;
};

} // namespace sqlite

class Storage;

/// A frame of a series (source/tit/data/storage.hpp FrameView).
class FrameView {
public:
  FrameView(Storage& storage, std::int64_t id) : storage_{&storage}, id_{id} {}
  auto id() const noexcept -> std::int64_t { return id_; }
  template<class T>
  void write_array(std::string name, std::span<const T> values) const;

private:
  Storage* storage_;
  std::int64_t id_;
};

/// A series of frames (source/tit/data/storage.hpp SeriesView).
class SeriesView {
public:
  SeriesView(Storage& storage, std::int64_t id)
      : storage_{&storage}, id_{id} {}
  auto id() const noexcept -> std::int64_t { return id_; }
  auto storage() const noexcept -> Storage& { return *storage_; }
  auto create_frame(double time) const -> FrameView;
  auto num_frames() const -> std::int64_t;

private:
  Storage* storage_;
  std::int64_t id_;
};

/// Particle storage in a .ttdb file (source/tit/data/storage.cpp:30-67).
class Storage {
public:
  using blob_type = ArrayBlob;

  explicit Storage(const std::filesystem::path& path) : db_{path} {
    db_.execute(R"SQL(
      PRAGMA journal_mode = WAL;
      PRAGMA foreign_keys = ON;
      CREATE TABLE IF NOT EXISTS Settings (
        id INTEGER PRIMARY KEY CHECK (id = 0),
        max_series INTEGER
      ) STRICT;
      INSERT OR IGNORE INTO Settings (id, max_series) VALUES (0, 5);
      CREATE TABLE IF NOT EXISTS DataSeries (
        id   INTEGER PRIMARY KEY AUTOINCREMENT,
        name TEXT NOT NULL
      ) STRICT;
      CREATE TABLE IF NOT EXISTS DataFrames (
        id        INTEGER PRIMARY KEY AUTOINCREMENT,
        series_id INTEGER NOT NULL,
        time      REAL NOT NULL,
        FOREIGN KEY (series_id) REFERENCES DataSeries(id) ON DELETE CASCADE
      ) STRICT;
      CREATE TABLE IF NOT EXISTS DataArrays (
        id       INTEGER PRIMARY KEY AUTOINCREMENT,
        frame_id INTEGER NOT NULL,
        name     TEXT NOT NULL,
        type     INTEGER,
        size     INTEGER,
        data     BLOB,
        FOREIGN KEY (frame_id) REFERENCES DataFrames(id) ON DELETE CASCADE
      ) STRICT;
    )SQL");
  }
  Storage(const Storage&) = delete;
  auto operator=(const Storage&) -> Storage& = delete;
  ~Storage() {
    try {
      wait();
    } catch (...) { // NOLINT: a failed background write cannot throw here
    }
  }

  auto max_series() -> std::int64_t {
    wait();
    return db_.run("SELECT max_series FROM Settings");
  }
  void set_max_series(std::int64_t value) {
    if (value <= 0) throw Exception{"Storage: max_series must be positive"};
    wait();
    db_.run("UPDATE Settings SET max_series = ?",
            [value](const sqlite::Api& a, void* s) { a.bind_int64(s, 1, value); });
    const std::int64_t extra = num_series() - value;
    if (extra > 0) {
      db_.run("DELETE FROM DataSeries WHERE id IN "
              "(SELECT id FROM DataSeries ORDER BY id ASC LIMIT ?)",
              [extra](const sqlite::Api& a, void* s) {
                a.bind_int64(s, 1, extra);
              });
    }
  }
  auto num_series() -> std::int64_t {
    wait();
    return db_.run("SELECT COUNT(*) FROM DataSeries");
  }

  /// New series; drops the oldest one when max_series are present.
  auto create_series(std::string_view name = "") -> SeriesView {
    wait();
    if (num_series() >= max_series()) {
      db_.run("DELETE FROM DataSeries WHERE id IN "
              "(SELECT id FROM DataSeries ORDER BY id ASC LIMIT 1)");
    }
    const std::string n{name};
    db_.run("INSERT INTO DataSeries (name) VALUES (?)",
            [&n](const sqlite::Api& a, void* s) {
              a.bind_text(s, 1, n.c_str(), -1, sqlite::transient());
            });
    return {*this, db_.last_insert_rowid()};
  }

  // ---- used by the views and by ParticleArray::write ----------------------
  auto create_frame_id(std::int64_t series, double time) -> std::int64_t {
    wait();
    return create_frame_id_(series, time);
  }
  auto series_num_frames(std::int64_t series) -> std::int64_t {
    wait();
    return db_.run("SELECT COUNT(*) FROM DataFrames WHERE series_id = ?",
                   [series](const sqlite::Api& a, void* s) {
                     a.bind_int64(s, 1, series);
                   });
  }
  void write_array(std::int64_t frame, const ArrayBlob& blob) {
    wait();
    write_array_(frame, blob);
  }

  /// Write a frame with its arrays on a background thread; returns at once.
  void write_frame_async(std::int64_t series, double time,
                         std::vector<ArrayBlob> arrays) {
    wait();
    pending_ = std::async(std::launch::async,
                          [this, series, time, a = std::move(arrays)] {
                            const std::int64_t f = create_frame_id_(series, time);
                            for (const ArrayBlob& b : a) write_array_(f, b);
                          });
  }

  /// Wait for a background write (rethrows its error).
  void wait() {
    if (pending_.valid()) pending_.get();
  }

private:
  auto create_frame_id_(std::int64_t series, double time) -> std::int64_t {
    const std::int64_t last_count =
        db_.run("SELECT COUNT(*) FROM DataFrames WHERE series_id = ? AND "
                "time >= ?",
                [series, time](const sqlite::Api& a, void* s) {
                  a.bind_int64(s, 1, series);
                  a.bind_double(s, 2, time);
                });
    if (last_count != 0) {
      throw Exception{"Storage: frame time must exceed the last frame's"};
    }
    db_.run("INSERT INTO DataFrames (series_id, time) VALUES (?, ?)",
            [series, time](const sqlite::Api& a, void* s) {
              a.bind_int64(s, 1, series);
              a.bind_double(s, 2, time);
            });
    return db_.last_insert_rowid();
  }

  void write_array_(std::int64_t frame, const ArrayBlob& blob) {
    if (blob.name.empty()) throw Exception{"Storage: empty array name"};
    const std::vector<std::byte> z = zstd_raw::encode(blob.bytes);
    db_.run("INSERT INTO DataArrays (frame_id, name, type, size, data) "
            "VALUES (?, ?, ?, ?, ?)",
            [&](const sqlite::Api& a, void* s) {
              a.bind_int64(s, 1, frame);
              a.bind_text(s, 2, blob.name.c_str(), -1, sqlite::transient());
              a.bind_int64(s, 3, blob.type);
              a.bind_int64(s, 4, blob.size);
              a.bind_blob64(s, 5, z.data(), z.size(), sqlite::transient());
            });
  }

  sqlite::Database db_;
  std::future<void> pending_;
};

inline auto SeriesView::create_frame(double time) const -> FrameView {
  return {*storage_, storage_->create_frame_id(id_, time)};
}
inline auto SeriesView::num_frames() const -> std::int64_t {
  return storage_->series_num_frames(id_);
}
template<class T>
void FrameView::write_array(std::string name, std::span<const T> values) const {
  storage_->write_array(id_, ArrayBlob::of<T>(std::move(name), values));
}

} // namespace tit::data

#endif // TITGPU_DATA_HPP
