// song_cli.cpp -- command-line driver with the reference's argv and output
// (main.cu:49-100), on top of the C ABI in include/song_gb300.h.
//
//   song build <build_data> <query_data> <search_top_k> <row> <dim> <return_top_k> <l2|ip|cos>
//   song test  <build_data> <query_data> <search_top_k> <row> <dim> <return_top_k> <l2|ip|cos>
//
// build: reads one-based LIBSVM vectors (parser.h:12-66), builds the graph
//        (graph.h:149-167) and writes bfsg.graph / bfsg.data in the working
//        directory (main.cu:78-85).
// test:  loads bfsg.graph / bfsg.data, reads the queries, searches them in one
//        batch (main.cu:23-35, 86-94) and prints the first return_top_k
//        zero-based ids of each query on one line, "%zu " per id.
//
// The reference bakes pq_size into the binary (fill_parameters.sh:12,35-53)
// and ignores search_top_k in GPU mode; here pq_size is search_top_k, or
// SONG_PQ_SIZE when set.  Graph constants follow KernelFixedDegreeGraph
// (kernelgraph.h:27-29: shift 5, degree 15, row capacity 31) unless
// SONG_SHIFT / SONG_SEARCH_DEGREE / SONG_FIXED_DEGREE are set.
// SONG_BUILD_DIV > 0 selects the batch-parallel build, SONG_BUILD_GPU=1 its
// searches on GPU 0 (the same graph).  Test mode starts at vertex 0, as the
// reference does, unless SONG_ENTRIES > 0: then each query starts from its
// SONG_STARTS (default 4) nearest of SONG_ENTRIES vertices drawn with seed
// SONG_ENTRY_SEED (default 11); SONG_COARSE > 0 makes the choice two-level
// with SONG_PROBES (default 4) clusters probed.  SONG_N_MULTIPROBE,
// SONG_FINISH_CNT and SONG_MULTIPROBE_DOUBLE_CHECK set the kernel's
// multi-probe knobs, which the reference fixes at build time
// (warp_astar_accelerator.h:29-30,307; fill_parameters.sh:36-37); defaults
// 1, 1 and 0, the reference's.
//
// Binary I/O (no reference counterpart; the reference parses LIBSVM text,
// parser.h:48-64): SONG_DATA_FORMAT=f32 makes build read <build_data> and
// SONG_QUERY_FORMAT=f32 makes test read <query_data> as raw little-endian
// float32 rows, the bfsg.data layout (the row count is the file size over
// 4 * dim); SONG_RESULTS=<file> makes test write nq x return_top_k
// little-endian uint64 ids (UINT64_MAX where a query has fewer) to <file>
// instead of printing the lines.
//
//   song convert <libsvm_in> <dim> <f32_out>
//
// writes a LIBSVM file's vectors as float32 rows, densified as test and build
// densify them.
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <thread>
#include <utility>
#include <vector>

#include "song_gb300.h"

namespace {

int env_int(const char *name, int dflt) {
  const char *v = getenv(name);
  return v && *v ? atoi(v) : dflt;
}

// parser.h:24-64: separators are ':' and ' '; pairs (index after a space,
// value after a colon); one-based indices; values read as double, stored as
// float.  Returns false on an unreadable file.
bool parse_libsvm(const char *path, int dim, std::vector<std::vector<std::pair<int, float>>> &rows,
                  std::string &err) {
  FILE *fp = fopen(path, "r");
  if (!fp) {
    err = std::string("File not found at (") + path + ")";
    return false;
  }
  const int MAX_LINE = 10000000;
  std::vector<char> buf(MAX_LINE);
  while (fgets(buf.data(), MAX_LINE, fp)) {
    std::vector<int> tok;
    for (int i = 0; buf[i] != '\0'; ++i)
      if (buf[i] == ':' || buf[i] == ' ') tok.push_back(i);
    std::vector<std::pair<int, float>> r;
    for (size_t i = 0; i + 1 < tok.size(); i += 2) {
      int index = 0;
      double v = 0;
      sscanf(buf.data() + tok[i] + 1, "%d", &index);
      sscanf(buf.data() + tok[i + 1] + 1, "%lf", &v);
      index -= 1;
      if (index < 0 || index >= dim) {
        fclose(fp);
        err = "feature index out of range in " + std::string(path);
        return false;
      }
      r.push_back(std::make_pair(index, static_cast<float>(v)));
    }
    rows.push_back(std::move(r));
  }
  fclose(fp);
  return true;
}

void densify(const std::vector<std::vector<std::pair<int, float>>> &rows, int dim, size_t n,
             std::vector<float> &out) {
  out.assign(n * static_cast<size_t>(dim), 0.0f);
  for (size_t i = 0; i < rows.size() && i < n; ++i)
    for (const auto &p : rows[i]) out[i * dim + p.first] = p.second;
}

// Raw little-endian float32 rows of dim floats; n = file size / (4 dim).
bool read_f32_rows(const char *path, int dim, std::vector<float> &out, size_t &n, std::string &err) {
  FILE *fp = fopen(path, "rb");
  if (!fp) {
    err = std::string("File not found at (") + path + ")";
    return false;
  }
  const size_t row_bytes = sizeof(float) * static_cast<size_t>(dim > 0 ? dim : 0);
  long long size = -1;
  if (fseek(fp, 0, SEEK_END) == 0) size = ftell(fp);
  if (dim <= 0 || size < 0 || fseek(fp, 0, SEEK_SET) != 0 || static_cast<size_t>(size) % row_bytes != 0) {
    fclose(fp);
    err = std::string(path) + ": size is not a whole number of rows of dim float32";
    return false;
  }
  n = static_cast<size_t>(size) / row_bytes;
  out.assign(n * static_cast<size_t>(dim), 0.0f);
  const size_t got = n ? fread(out.data(), row_bytes, n, fp) : 0;
  fclose(fp);
  if (got != n) {
    err = std::string(path) + ": short read";
    return false;
  }
  return true;
}

// SONG_DATA_FORMAT / SONG_QUERY_FORMAT: "libsvm" (default) or "f32"; -1 otherwise.
int input_format(const char *name) {
  const char *v = getenv(name);
  if (!v || !*v || strcmp(v, "libsvm") == 0) return 0;
  return strcmp(v, "f32") == 0 ? 1 : -1;
}

// The rows of a LIBSVM or float32 file; with rows >= 0 zero-padded or cut to
// that many (build densifies to <row>), else all of them.
bool read_rows(const char *path, int dim, int format, long long rows, std::vector<float> &out, size_t &n,
               std::string &err) {
  if (format == 1) {
    if (!read_f32_rows(path, dim, out, n, err)) return false;
  } else {
    std::vector<std::vector<std::pair<int, float>>> sparse;
    if (!parse_libsvm(path, dim, sparse, err)) return false;
    n = sparse.size();
    densify(sparse, dim, n, out);
  }
  if (rows >= 0) {
    out.resize(static_cast<size_t>(rows) * static_cast<size_t>(dim), 0.0f);
    n = static_cast<size_t>(rows);
  }
  return true;
}

void usage(char **argv) {
  printf("Usage: %s <build/test> <build_data> <query_data> <search_top_k> <row> <dim> <return_top_k> <l2/ip/cos>\n"
         "       %s convert <libsvm_in> <dim> <f32_out>\n",
         argv[0], argv[0]);
}

}  // namespace

// count distinct ids of 0..n-1 in draw order: a partial Fisher-Yates shuffle
// driven by splitmix64 from `seed` (any prefix is a uniform sample).
std::vector<uint64_t> sample_ids(uint64_t n, int count, uint64_t seed) {
  if (static_cast<uint64_t>(count) > n) count = static_cast<int>(n);
  std::vector<uint64_t> perm(n);
  for (uint64_t i = 0; i < n; ++i) perm[i] = i;
  uint64_t x = seed;
  for (int i = 0; i < count; ++i) {
    x += 0x9E3779B97F4A7C15ull;
    uint64_t z = x;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    const uint64_t j = static_cast<uint64_t>(i) + z % (n - static_cast<uint64_t>(i));
    std::swap(perm[i], perm[j]);
  }
  perm.resize(static_cast<size_t>(count));
  return perm;
}

int main(int argc, char **argv) {
  if (argc == 5 && strcmp(argv[1], "convert") == 0) {
    const int dim = atoi(argv[3]);
    std::string err = "dim must be positive";
    std::vector<float> v;
    size_t n = 0;
    if (dim <= 0 || !read_rows(argv[2], dim, 0, -1, v, n, err)) {
      fprintf(stderr, "%s\n", err.c_str());
      return 1;
    }
    FILE *fo = fopen(argv[4], "wb");
    bool ok = fo && (n == 0 || fwrite(v.data(), sizeof(float) * dim, n, fo) == n);
    if (fo && fclose(fo) != 0) ok = false;
    if (!ok) {
      fprintf(stderr, "cannot write %s\n", argv[4]);
      return 1;
    }
    return 0;
  }
  if (argc != 9) {
    usage(argv);
    return 1;
  }
  const uint64_t row = strtoull(argv[5], nullptr, 10);
  const int dim = atoi(argv[6]);
  const int display = atoi(argv[7]);
  const std::string dt = argv[8];
  int metric;
  if (dt == "l2") metric = SONG_METRIC_L2;
  else if (dt == "ip") metric = SONG_METRIC_IP;
  else if (dt == "cos") metric = SONG_METRIC_COS;
  else {
    usage(argv);
    return 1;
  }
  const std::string mode = argv[1];
  const int shift = env_int("SONG_SHIFT", 5);
  const int search_degree = env_int("SONG_SEARCH_DEGREE", 15);
  const int fixed_degree = env_int("SONG_FIXED_DEGREE", (1 << shift) - 1);
  std::string err;
  if (mode == "build") {
    const int fmt = input_format("SONG_DATA_FORMAT");
    std::vector<float> data;
    size_t n_read = 0;
    if (fmt < 0) err = "SONG_DATA_FORMAT must be libsvm or f32";
    if (fmt < 0 || !read_rows(argv[2], dim, fmt, static_cast<long long>(row), data, n_read, err)) {
      fprintf(stderr, "%s\n", err.c_str());
      return 1;
    }
    std::vector<uint64_t> graph(static_cast<size_t>(row) << shift);
    fprintf(stderr, "Writing the graph and data...");
    const int nthreads = static_cast<int>(std::thread::hardware_concurrency());
    int rc = env_int("SONG_BUILD_GPU", 0)
                 ? song_graph_build_gpu(data.data(), row, dim, metric, shift, search_degree, fixed_degree, 150,
                                        env_int("SONG_BUILD_DIV", 0), 0, nthreads, graph.data())
                 : song_graph_build(data.data(), row, dim, metric, shift, search_degree, fixed_degree, 150,
                                    env_int("SONG_BUILD_DIV", 0), nthreads, graph.data());
    if (rc) {
      fprintf(stderr, "\n%s: %s\n", song_status_string(rc), song_last_error());
      return 1;
    }
    FILE *fd = fopen("bfsg.data", "wb");
    FILE *fg = fopen("bfsg.graph", "wb");
    if (!fd || !fg) {
      fprintf(stderr, "\ncannot write bfsg.data / bfsg.graph\n");
      return 1;
    }
    fwrite(data.data(), sizeof(float), data.size(), fd);
    fwrite(graph.data(), sizeof(uint64_t), graph.size(), fg);
    fclose(fd);
    fclose(fg);
    fprintf(stderr, "done\n");
    return 0;
  }
  if (mode == "test") {
    fprintf(stderr, "Loading the graph and data...");
    song_index *ix = nullptr;
    int rc = song_index_load("bfsg.graph", "bfsg.data", row, dim, shift, metric, SONG_STORAGE_F32, 0, &ix);
    if (rc) {
      fprintf(stderr, "\n%s: %s\n", song_status_string(rc), song_last_error());
      return 1;
    }
    fprintf(stderr, "done\n");
    const int fmt = input_format("SONG_QUERY_FORMAT");
    std::vector<float> q;
    size_t n_q = 0;
    if (fmt < 0) err = "SONG_QUERY_FORMAT must be libsvm or f32";
    if (fmt < 0 || !read_rows(argv[3], dim, fmt, -1, q, n_q, err) || n_q > 0x7fffffff) {
      fprintf(stderr, "%s\n", n_q > 0x7fffffff ? "too many queries" : err.c_str());
      song_index_free(ix);
      return 1;
    }
    const int pq = env_int("SONG_PQ_SIZE", atoi(argv[4]));
    const int n_entries = env_int("SONG_ENTRIES", 0);
    if (n_entries > 0) {
      const std::vector<uint64_t> ent = sample_ids(row, n_entries, static_cast<uint64_t>(env_int("SONG_ENTRY_SEED", 11)));
      const int coarse = env_int("SONG_COARSE", 0);
      rc = coarse > 0 ? song_index_set_entries_2level(ix, ent.data(), static_cast<int>(ent.size()), coarse,
                                                      env_int("SONG_PROBES", 4), env_int("SONG_STARTS", 4))
                      : song_index_set_entries(ix, ent.data(), static_cast<int>(ent.size()), env_int("SONG_STARTS", 4));
      if (rc) {
        fprintf(stderr, "%s: %s\n", song_status_string(rc), song_last_error());
        song_index_free(ix);
        return 1;
      }
    }
    const int probes = env_int("SONG_N_MULTIPROBE", 1), finish_cnt = env_int("SONG_FINISH_CNT", 1);
    const int double_check = env_int("SONG_MULTIPROBE_DOUBLE_CHECK", 0);
    if (probes != 1 || finish_cnt != 1 || double_check != 0) {
      rc = song_index_set_multiprobe(ix, probes, finish_cnt, double_check);
      if (rc) {
        fprintf(stderr, "%s: %s\n", song_status_string(rc), song_last_error());
        song_index_free(ix);
        return 1;
      }
    }
    const int nq = static_cast<int>(n_q);
    std::vector<uint64_t> out(static_cast<size_t>(nq) * pq);
    rc = song_search(ix, q.data(), nq, pq, pq, out.data(), nullptr, nullptr);
    song_index_free(ix);
    if (rc) {
      fprintf(stderr, "%s: %s\n", song_status_string(rc), song_last_error());
      return 1;
    }
    const char *results = getenv("SONG_RESULTS");
    if (results && *results) {
      const int show = display > 0 ? display : 0;
      std::vector<uint64_t> ids(static_cast<size_t>(nq) * show, UINT64_MAX);
      for (int i = 0; i < nq; ++i)
        for (int j = 0; j < pq && j < show; ++j) ids[static_cast<size_t>(i) * show + j] = out[static_cast<size_t>(i) * pq + j];
      FILE *fo = fopen(results, "wb");
      bool ok = fo && (ids.empty() || fwrite(ids.data(), sizeof(uint64_t), ids.size(), fo) == ids.size());
      if (fo && fclose(fo) != 0) ok = false;
      if (!ok) {
        fprintf(stderr, "cannot write %s\n", results);
        return 1;
      }
      return 0;
    }
    for (int i = 0; i < nq; ++i) {
      for (int j = 0; j < pq && j < display; ++j) {
        uint64_t id = out[static_cast<size_t>(i) * pq + j];
        if (id == UINT64_MAX) break;
        printf("%zu ", static_cast<size_t>(id));
      }
      printf("\n");
    }
    return 0;
  }
  usage(argv);
  return 1;
}
