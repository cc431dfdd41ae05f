// abm -- the command-line driver of ParAGraph's agent-based citation model, on the GB300 engine.
//
// Drop-in for the reference's `abm` executable (src/main.cu:22-175 with execute(),
// src/kernel.cu:1592-1948): the same options and defaults, the same input files (edge list, node
// list, out-degree bag, recency probabilities, planted papers) and the same outputs (edge list,
// auxiliary per-node attributes, log file).  Each epoch is one pg_grow_epoch (or pg_er_epoch) on
// the device through the C ABI in include/paragraph_gb300.h; the host only parses, maps ids and
// writes files.
//
// Options of the reference (src/main.cu:29-114):
//   --edgelist --nodelist --out-degree-bag --recency-probabilities --growth-rate --num-cycles
//   --same-year-proportion --output-file --auxiliary-information-file --log-file   (required)
//   --planted-nodes --preferential-weight --recency-weight --fitness-weight --alpha
//   --fully-random-citations --num-processors --log-level
//   --use-warp-bfs --use-batching --use-multistage-kernel --max-batch-size
//     (accepted for compatibility; the device step has one persistent kernel per stage and no
//      host mini-batches, so they do not change anything)
// Options of the reference's ER branch (results/slurm-8640738.out:555-557):
//   --model {pa,er-gnp}  --er-probability P  --er-edges-per-node K (P = K / n each epoch)
// Options added here:
//   --seed S                       Philox key (the reference seeds from the clock)
//   --weight-model {refcompat,baseline}
//                                  refcompat (default): the reference's own linear score model;
//                                  baseline: w_j = f_j^gamma (indeg_j+1)^pa_alpha
//                                  exp(-(t-t_j)/tau) beta^[j in 2-hop ball of the anchors]
//   --pa-alpha --tau --gamma --beta --num-anchors --mean-out-degree   (baseline parameters)
//   --sampler {thinning,enumerate} (baseline)   --device D
//   --output-nodelist FILE         node list (id, year) of the grown graph, so it can seed a run
//   --epoch-log FILE               one JSON line per epoch (edges, device ms, bytes, edges/s)
//
// Output formats (Graph::WriteGraph / WriteAttributes, src/graph.cu:909-1211): "#source,target"
// then one "source,target" row per edge with original ids, rows grouped by source in ascending
// sequence id and targets ascending; new papers take ids max(original id)+1, +2, ...  The
// attribute file has the reference's 15 columns; seeds print -1 for the agent-only fields and
// "no_generators".  (The reference's WriteGraph reuses one digit buffer for source and target, so
// after a source's first edge it prints target digits as the source; this writer prints the
// source id on every row.)
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <sstream>
#include <string>
#include <vector>

#include "paragraph_gb300.h"

namespace {

struct Options {
    std::map<std::string, std::string> kv;
    bool has(const std::string& k) const { return kv.count(k) != 0; }
    std::string str(const std::string& k, const std::string& d = "") const {
        auto it = kv.find(k);
        return it == kv.end() ? d : it->second;
    }
    double num(const std::string& k, double d) const {
        auto it = kv.find(k);
        return it == kv.end() ? d : std::stod(it->second);
    }
    bool flag(const std::string& k, bool d) const {
        auto it = kv.find(k);
        if (it == kv.end()) return d;
        return it->second == "true" || it->second == "1" || it->second == "yes";
    }
};

const char* kKnown[] = {
    "--edgelist", "--nodelist", "--out-degree-bag", "--recency-probabilities", "--use-warp-bfs",
    "--use-batching", "--use-multistage-kernel", "--max-batch-size", "--planted-nodes",
    "--preferential-weight", "--recency-weight", "--fitness-weight", "--alpha",
    "--fully-random-citations", "--growth-rate", "--num-cycles", "--same-year-proportion",
    "--output-file", "--auxiliary-information-file", "--log-file", "--num-processors", "--log-level",
    "--model", "--er-probability", "--er-edges-per-node", "--seed", "--weight-model", "--pa-alpha",
    "--tau", "--gamma", "--beta", "--num-anchors", "--mean-out-degree", "--sampler", "--device",
    "--output-nodelist", "--epoch-log"};
const char* kRequired[] = {"--edgelist", "--nodelist", "--growth-rate", "--num-cycles",
                           "--output-file", "--auxiliary-information-file", "--log-file"};

void usage() {
    std::fprintf(stderr,
                 "Usage: abm --edgelist FILE --nodelist FILE --out-degree-bag FILE\n"
                 "           --recency-probabilities FILE --growth-rate R --num-cycles N\n"
                 "           --same-year-proportion P --output-file FILE\n"
                 "           --auxiliary-information-file FILE --log-file FILE [options]\n"
                 "Agent Based Modelling of citation-graph growth on one GB300.\n");
}

bool parse(int argc, char** argv, Options& o, std::string& err) {
    for (int i = 1; i < argc; ++i) {
        std::string a = argv[i];
        if (a == "-h" || a == "--help") {
            err = "help";
            return false;
        }
        std::string v;
        const size_t eq = a.find('=');
        if (eq != std::string::npos) {
            v = a.substr(eq + 1);
            a = a.substr(0, eq);
        } else {
            if (i + 1 >= argc) {
                err = "missing value for " + a;
                return false;
            }
            v = argv[++i];
        }
        bool known = false;
        for (const char* k : kKnown) known |= a == k;
        if (!known) {
            err = "unknown option " + a;
            return false;
        }
        o.kv[a] = v;
    }
    const bool er = o.str("--model", "pa") == "er-gnp";
    for (const char* k : kRequired)
        if (!o.has(k)) {
            err = std::string(k) + " is required";
            return false;
        }
    if (!er) {
        if (!o.has("--same-year-proportion")) {
            err = "--same-year-proportion is required";
            return false;
        }
        if (o.str("--weight-model", "refcompat") == "refcompat" &&
            (!o.has("--out-degree-bag") || !o.has("--recency-probabilities"))) {
            err = "--out-degree-bag and --recency-probabilities are required";
            return false;
        }
    }
    return true;
}

// The reference's delimiter rule (Graph::get_delimiter, includes/graph.cuh:41-53): the first of
// ',', tab, space found in the first line.
char delimiter_of(const std::string& path) {
    std::ifstream f(path);
    std::string line;
    std::getline(f, line);
    if (line.find(',') != std::string::npos) return ',';
    if (line.find('\t') != std::string::npos) return '\t';
    if (line.find(' ') != std::string::npos) return ' ';
    return ',';
}

bool read_rows(const std::string& path, std::vector<std::vector<std::string>>& rows, std::string& err) {
    std::ifstream f(path);
    if (!f) {
        err = "cannot open " + path;
        return false;
    }
    const char d = delimiter_of(path);
    std::string line;
    while (std::getline(f, line)) {
        if (!line.empty() && line.back() == '\r') line.pop_back();
        if (line.empty() || line[0] == '#') continue;
        std::vector<std::string> cols;
        std::stringstream ss(line);
        std::string c;
        while (std::getline(ss, c, d)) cols.push_back(c);
        rows.push_back(std::move(cols));
    }
    return true;
}

struct Logger {
    std::ofstream f;
    int level = 0;  // 0 silent, 1 info, 2 debug (the reference's --log-level)
    std::chrono::steady_clock::time_point t0 = std::chrono::steady_clock::now();
    void write(const char* kind, int lvl, const std::string& msg) {
        if (level < lvl || !f) return;
        const auto s = std::chrono::duration_cast<std::chrono::seconds>(std::chrono::steady_clock::now() - t0).count();
        const long long d = s / 86400, h = (s / 3600) % 24, m = (s / 60) % 60, sec = s % 60;
        f << kind << "[" << d << "-" << h << ":" << m << ":" << sec << "](t=" << s << "s) " << msg << '\n';
        f.flush();
    }
    void info(const std::string& m) { write("[INFO]", 1, m); }
    void debug(const std::string& m) { write("[DEBUG]", 2, m); }
    void error(const std::string& m) { write("[ERROR]", 0, m); }
};

int die(Logger& log, const std::string& msg) {
    std::fprintf(stderr, "abm: %s\n", msg.c_str());
    log.error(msg);
    return 1;
}

#define PG_TRY(ctx, call)                                                                          \
    do {                                                                                           \
        const pg_status st_ = (call);                                                              \
        if (st_ != PG_OK)                                                                          \
            return die(log, std::string(#call) + ": " + pg_status_string(st_) + ": " +            \
                                (ctx ? pg_last_error(ctx) : ""));                                  \
    } while (0)

uint64_t splitmix(uint64_t& s) {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

int run(int argc, char** argv);

}  // namespace

// Malformed numbers in the options or the input files end the run with a message, not an abort.
int main(int argc, char** argv) {
    try {
        return run(argc, argv);
    } catch (const std::exception& e) {
        std::fprintf(stderr, "abm: malformed number or input (%s)\n", e.what());
        return 1;
    }
}

namespace {

int run(int argc, char** argv) {
    Options o;
    std::string perr;
    Logger log;
    if (!parse(argc, argv, o, perr)) {
        usage();
        if (perr == "help") return 0;
        std::fprintf(stderr, "abm: %s\n", perr.c_str());
        return 1;
    }
    log.f.open(o.str("--log-file"));
    log.level = (int)o.num("--log-level", 1);
    const bool er = o.str("--model", "pa") == "er-gnp";
    const std::string wm = o.str("--weight-model", "refcompat");
    if (!er && wm != "refcompat" && wm != "baseline") return die(log, "--weight-model must be refcompat or baseline");
    const bool rc = !er && wm == "refcompat";
    const double growth = o.num("--growth-rate", 0.0);
    const int cycles = (int)o.num("--num-cycles", 0);
    const uint64_t seed = (uint64_t)o.num("--seed", 42);
    if (!(growth > 0.0) || cycles < 1) return die(log, "--growth-rate must be > 0 and --num-cycles >= 1");

    // ---- node list: (node, year); sequence ids follow ascending original id (ParseNodelist,
    // src/graph.cu:336-374)
    std::vector<std::vector<std::string>> rows;
    if (!read_rows(o.str("--nodelist"), rows, perr)) return die(log, perr);
    std::map<int64_t, int32_t> year_of;
    for (const auto& r : rows) {
        if (r.size() < 2) return die(log, "nodelist rows need (node, year)");
        year_of[std::stoll(r[0])] = (int32_t)std::stol(r[1]);
    }
    if (year_of.size() < 2) return die(log, "the node list needs at least two nodes");
    std::vector<int64_t> orig;  // sequence id -> original id
    std::map<int64_t, int32_t> seq_of;
    std::vector<int32_t> pub;
    int32_t max_year = INT32_MIN;
    for (const auto& [id, y] : year_of) {
        seq_of[id] = (int32_t)orig.size();
        orig.push_back(id);
        pub.push_back(y);
        max_year = std::max(max_year, y);
    }
    const int64_t n0 = (int64_t)orig.size();
    // ---- edge list: both ends must be listed nodes (ParseEdgelist, src/graph.cu:376-447)
    rows.clear();
    if (!read_rows(o.str("--edgelist"), rows, perr)) return die(log, perr);
    std::vector<int32_t> src, dst;
    for (const auto& r : rows) {
        if (r.size() < 2) continue;
        auto a = seq_of.find(std::stoll(r[0])), b = seq_of.find(std::stoll(r[1]));
        if (a == seq_of.end() || b == seq_of.end()) continue;
        src.push_back(a->second);
        dst.push_back(b->second);
    }
    log.info("read " + std::to_string(n0) + " nodes and " + std::to_string(src.size()) + " edges");

    // ---- model inputs
    std::vector<int32_t> bag;
    std::vector<double> rec;
    struct Plant {
        int line, lag, peak, dur, count;
    };
    std::map<int, std::vector<Plant>> planted;  // cycle index (1-based) -> lines
    if (rc) {
        rows.clear();
        if (!read_rows(o.str("--out-degree-bag"), rows, perr)) return die(log, perr);
        for (const auto& r : rows)
            if (r.size() >= 2) bag.push_back((int32_t)std::stol(r[1]));
        if (bag.empty()) return die(log, "the out-degree bag is empty");
        rows.clear();
        if (!read_rows(o.str("--recency-probabilities"), rows, perr)) return die(log, perr);
        for (const auto& r : rows) {
            if (r.size() < 2) continue;
            const long age = std::stol(r[0]);
            if (age < 0 || age >= 1024) continue;
            if ((size_t)age >= rec.size()) rec.resize((size_t)age + 1, 0.0);
            rec[(size_t)age] = std::stod(r[1]);
        }
        if (o.has("--planted-nodes") && !o.str("--planted-nodes").empty()) {
            rows.clear();
            if (!read_rows(o.str("--planted-nodes"), rows, perr)) return die(log, perr);
            int line = 0;
            for (const auto& r : rows) {
                if (r.size() < 5) continue;
                planted[std::stoi(r[0])].push_back(
                    {line, std::stoi(r[1]), std::stoi(r[2]), std::stoi(r[3]), std::stoi(r[4])});
                ++line;
            }
        }
    }

    // ---- seed fitness: refcompat peak values from the reference's power law (InitializeFitness,
    // src/abm.cu:124-150); baseline lognormal(0, 1).  Both from a seeded host generator.
    std::vector<float> fit((size_t)n0);
    uint64_t hs = seed ^ 0x5EEDF17ull;
    if (rc) {
        std::vector<uint64_t> tab(1000);
        pg_rc_fitness_table(tab.data());
        for (int64_t i = 0; i < n0; ++i) {
            const uint64_t u = splitmix(hs);
            int v = 1000;
            for (int k = 0; k < 1000; ++k)
                if (u < tab[(size_t)k]) {
                    v = k + 1;
                    break;
                }
            fit[(size_t)i] = (float)v;
        }
    } else {
        for (int64_t i = 0; i < n0; ++i) {
            double u1 = ((double)(splitmix(hs) >> 11) + 1.0) * 0x1p-53, u2 = (double)(splitmix(hs) >> 11) * 0x1p-53;
            fit[(size_t)i] = (float)std::exp(std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2));
        }
    }

    // ---- device context
    pg_config cfg{};
    cfg.device = (int32_t)o.num("--device", 0);
    cfg.num_replicas = 1;
    cfg.seed = seed;
    cfg.weight_model = rc ? PG_WEIGHTS_REFCOMPAT : PG_WEIGHTS_BASELINE;
    cfg.record_trace = 1;  // anchors / arrivals for the attribute file
    cfg.sampler = o.str("--sampler", "thinning") == "enumerate" ? PG_SAMPLER_ENUMERATE : PG_SAMPLER_THINNING;
    pg_ctx* ctx = nullptr;
    {
        const pg_status st = pg_create(&ctx, &cfg);
        if (st != PG_OK) return die(log, std::string("pg_create: ") + pg_status_string(st) + ": " + (ctx ? pg_last_error(ctx) : ""));
    }
    PG_TRY(ctx, pg_load_graph(ctx, n0, pub.data(), fit.data(), (int64_t)src.size(), src.data(), dst.data()));
    pg_pa_params prm;
    pg_default_params(&prm);
    prm.growth_rate = growth;
    prm.fixed_new_nodes = 0;
    if (!rc) {
        prm.alpha = o.num("--pa-alpha", 1.0);
        prm.tau = o.num("--tau", 5.0);
        prm.gamma = o.num("--gamma", 1.0);
        prm.beta = o.num("--beta", 4.0);
        prm.num_anchors = (int32_t)o.num("--num-anchors", 3);
        prm.mean_out_degree = o.num("--mean-out-degree", 15.0);
    }
    PG_TRY(ctx, pg_set_params(ctx, 0, &prm));
    const int32_t start_year = max_year + 1;
    PG_TRY(ctx, pg_set_epoch(ctx, start_year));
    if (rc) {
        pg_rc_params rp{};
        rp.pa_weight = o.num("--preferential-weight", -1.0);
        rp.rec_weight = o.num("--recency-weight", -1.0);
        rp.fit_weight = o.num("--fitness-weight", -1.0);
        rp.alpha = o.num("--alpha", -1.0);
        rp.fully_random = o.num("--fully-random-citations", 0.05);
        rp.same_year = o.num("--same-year-proportion", 0.0);
        rp.growth_rate = growth;
        rp.gamma = 3;
        rp.decay = 3;
        PG_TRY(ctx, pg_rc_configure(ctx, 0, &rp, bag.data(), (int64_t)bag.size(), rec.data(), (int32_t)rec.size()));
    }

    // ---- per-node attributes kept on the host for the attribute file
    std::vector<int32_t> lag((size_t)n0, 0), dur((size_t)n0, 1000), plant_line((size_t)n0, -1), gen((size_t)n0, -1),
        assigned((size_t)n0, -1);
    std::vector<double> wpa((size_t)n0, -1.0), wrec((size_t)n0, -1.0), wfit((size_t)n0, -1.0), walpha((size_t)n0, -1.0);
    // generators of each agent as sequence ids, up to 4 (the anchors of the baseline model, the
    // generator of refcompat), -1 unused
    std::vector<int32_t> gens((size_t)n0 * 4, -1);
    std::ofstream elog;
    if (o.has("--epoch-log")) elog.open(o.str("--epoch-log"));
    log.info("start year " + std::to_string(start_year) + ", " + std::to_string(cycles) + " cycles, model " +
             (er ? std::string("er-gnp") : wm));
    if (er) {
        // size the arena for every cycle up front: a PA plan does not cover ER edge counts, and an
        // arena outgrown mid-run is rebuilt through the host
        int64_t n = 0, m = 0;
        pg_get_counts(ctx, 0, &n, &m);
        double nf = (double)n, mf = (double)m;
        for (int cyc = 0; cyc < cycles; ++cyc) {
            const double nn = std::ceil(nf * growth);
            double p = o.num("--er-probability", -1.0);
            if (o.has("--er-edges-per-node")) p = o.num("--er-edges-per-node", 0.0) / nf;
            p = std::min(std::max(p, 0.0), 1.0);
            const double mu = nn * nf * p;
            mf += mu + 8.0 * std::sqrt(mu) + 1024.0;
            nf += nn;
        }
        PG_TRY(ctx, pg_reserve(ctx, (int64_t)nf, (int64_t)mf));
    }
    const auto t_run = std::chrono::steady_clock::now();
    int64_t total_edges = 0;
    for (int cyc = 0; cyc < cycles; ++cyc) {
        int64_t n = 0, m = 0, nn = 0, ne = 0;
        pg_get_counts(ctx, 0, &n, &m);
        if (er) {
            nn = (int64_t)std::ceil((double)n * growth);
            double p = o.num("--er-probability", -1.0);
            if (o.has("--er-edges-per-node")) p = o.num("--er-edges-per-node", 0.0) / (double)n;
            if (!(p >= 0.0 && p <= 1.0)) return die(log, "--er-probability must be in [0, 1]");
            PG_TRY(ctx, pg_er_epoch(ctx, nn, p, &ne));
        } else {
            PG_TRY(ctx, pg_grow_epoch(ctx, &nn, &ne));
        }
        total_edges += ne;
        // per-paper draws of the new papers
        gen.resize((size_t)(n + nn), -1);
        assigned.resize((size_t)(n + nn), -1);
        wpa.resize((size_t)(n + nn), -1.0);
        wrec.resize((size_t)(n + nn), -1.0);
        wfit.resize((size_t)(n + nn), -1.0);
        walpha.resize((size_t)(n + nn), -1.0);
        lag.resize((size_t)(n + nn), 0);
        dur.resize((size_t)(n + nn), 1000);
        plant_line.resize((size_t)(n + nn), -1);
        gens.resize((size_t)(n + nn) * 4, -1);
        if (rc) {
            std::vector<double> ag((size_t)nn * 6);
            PG_TRY(ctx, pg_rc_copy_agents(ctx, 0, ag.data()));
            for (int64_t a = 0; a < nn; ++a) {
                const size_t v = (size_t)(n + a);
                wpa[v] = ag[(size_t)a * 6 + 0];
                wrec[v] = ag[(size_t)a * 6 + 1];
                wfit[v] = ag[(size_t)a * 6 + 2];
                walpha[v] = ag[(size_t)a * 6 + 3];
                gen[v] = (int32_t)ag[(size_t)a * 6 + 4];
                gens[v * 4] = gen[v];
                assigned[v] = (int32_t)ag[(size_t)a * 6 + 5];
            }
            // planted papers of this cycle (ABM::PlantNodes, includes/abm.cuh:486-504)
            auto it = planted.find(cyc + 1);
            if (it != planted.end()) {
                int64_t done = 0;
                for (const Plant& pl : it->second) {
                    const int64_t cnt = std::min<int64_t>(pl.count, nn - done);
                    if (cnt <= 0) break;
                    std::vector<int32_t> L((size_t)cnt, pl.lag), P((size_t)cnt, pl.peak), D((size_t)cnt, pl.dur);
                    PG_TRY(ctx, pg_rc_set_nodes(ctx, 0, n + done, cnt, L.data(), P.data(), D.data()));
                    for (int64_t i = 0; i < cnt; ++i) {
                        lag[(size_t)(n + done + i)] = pl.lag;
                        dur[(size_t)(n + done + i)] = pl.dur;
                        plant_line[(size_t)(n + done + i)] = pl.line;
                    }
                    done += cnt;
                }
            }
        } else if (!er) {
            std::vector<int32_t> anc((size_t)nn * 4);
            PG_TRY(ctx, pg_copy_anchors(ctx, 0, anc.data()));
            for (int64_t a = 0; a < nn; ++a) gen[(size_t)(n + a)] = anc[(size_t)a * 4];
            std::copy(anc.begin(), anc.end(), gens.begin() + (ptrdiff_t)(n * 4));
        }
        pg_stats st{};
        pg_get_stats(ctx, &st);
        log.info("cycle " + std::to_string(cyc + 1) + ": " + std::to_string(nn) + " new papers, " +
                 std::to_string(ne) + " new edges, device " + std::to_string(st.ms_total) + " ms");
        if (elog) {
            char buf[512];
            std::snprintf(buf, sizeof(buf),
                          "{\"cycle\": %d, \"year\": %d, \"nodes\": %lld, \"new_nodes\": %lld, \"new_edges\": %lld, "
                          "\"ms_device\": %.4f, \"bytes_alg\": %lld, \"edges_per_s\": %.1f}\n",
                          cyc + 1, start_year + cyc, (long long)(n + nn), (long long)nn, (long long)ne, st.ms_total,
                          (long long)st.bytes_alg, st.ms_total > 0 ? ne / (st.ms_total * 1e-3) : 0.0);
            elog << buf;
        }
    }
    const double run_s = std::chrono::duration<double>(std::chrono::steady_clock::now() - t_run).count();

    // ---- outputs
    int64_t n = 0, m = 0;
    pg_get_counts(ctx, 0, &n, &m);
    int64_t next_id = orig.back() + 1;
    while ((int64_t)orig.size() < n) orig.push_back(next_id++);
    std::vector<int64_t> off((size_t)n + 1);
    std::vector<int32_t> col((size_t)std::max<int64_t>(m, 1));
    PG_TRY(ctx, pg_copy_csr(ctx, 0, 0, off.data(), col.data()));
    std::vector<int32_t> indeg((size_t)n), outdeg((size_t)n), pubs((size_t)n);
    std::vector<float> fits((size_t)n);
    PG_TRY(ctx, pg_copy_degrees(ctx, 0, indeg.data(), outdeg.data()));
    PG_TRY(ctx, pg_copy_nodes(ctx, 0, pubs.data(), fits.data()));
    {
        // the edge rows are formatted on the device (pg_format_edges) and written in one block
        FILE* f = std::fopen(o.str("--output-file").c_str(), "wb");
        if (!f) return die(log, "cannot write " + o.str("--output-file"));
        std::fputs("#source,target\n", f);
        int64_t bytes = 0;
        PG_TRY(ctx, pg_format_edges(ctx, 0, orig.data(), n, nullptr, 0, &bytes));
        std::vector<char> txt((size_t)std::max<int64_t>(bytes, 1));
        PG_TRY(ctx, pg_format_edges(ctx, 0, orig.data(), n, txt.data(), bytes, &bytes));
        std::fwrite(txt.data(), 1, (size_t)bytes, f);
        std::fclose(f);
    }
    {
        FILE* f = std::fopen(o.str("--auxiliary-information-file").c_str(), "wb");
        if (!f) return die(log, "cannot write " + o.str("--auxiliary-information-file"));
        std::fputs("node_id,type,year,pa_weight,rec_weight,fit_weight,fit_lag_duration,fit_peak_value,"
                   "fit_peak_duration,alpha,in_degree,out_degree,assigned_out_degree,"
                   "planted_nodes_line_number,generator_node_string\n",
                   f);
        // the rows are formatted on the device (pg_format_attributes): the per-paper columns go
        // up, year, fitness and degrees are the arena's own
        std::vector<double> draws((size_t)n * 4);
        std::vector<int32_t> ints((size_t)n * 4);
        std::vector<int64_t> gid((size_t)n * 4, -1);
        for (int64_t v = 0; v < n; ++v) {
            const size_t u = (size_t)v;
            const bool agent = v >= n0;
            draws[u * 4 + 0] = agent ? wpa[u] : -1.0;
            draws[u * 4 + 1] = agent ? wrec[u] : -1.0;
            draws[u * 4 + 2] = agent ? wfit[u] : -1.0;
            draws[u * 4 + 3] = agent ? walpha[u] : -1.0;
            ints[u * 4 + 0] = rc ? lag[u] : -1;
            ints[u * 4 + 1] = rc ? dur[u] : -1;
            ints[u * 4 + 2] = agent ? (rc ? assigned[u] : outdeg[u]) : -1;
            ints[u * 4 + 3] = agent ? plant_line[u] : -1;
            for (int i = 0; agent && i < 4; ++i) {
                const int32_t x = gens[u * 4 + (size_t)i];
                if (x >= 0) gid[u * 4 + (size_t)i] = orig[(size_t)x];
            }
        }
        pg_attr_rows rows{};
        rows.num_nodes = n;
        rows.num_seed = n0;
        rows.ids = orig.data();
        rows.draws = draws.data();
        rows.ints = ints.data();
        rows.generators = gid.data();
        rows.peak_integer = rc ? 1 : 0;  // refcompat: the integer peak; else the fp32 fitness, "%.9g"
        int64_t bytes = 0;
        PG_TRY(ctx, pg_format_attributes(ctx, 0, &rows, nullptr, 0, &bytes));
        std::vector<char> txt((size_t)std::max<int64_t>(bytes, 1));
        PG_TRY(ctx, pg_format_attributes(ctx, 0, &rows, txt.data(), bytes, &bytes));
        std::fwrite(txt.data(), 1, (size_t)bytes, f);
        std::fclose(f);
    }
    if (o.has("--output-nodelist")) {
        FILE* f = std::fopen(o.str("--output-nodelist").c_str(), "wb");
        if (!f) return die(log, "cannot write " + o.str("--output-nodelist"));
        std::fputs("#node,year\n", f);
        for (int64_t v = 0; v < n; ++v) std::fprintf(f, "%lld,%d\n", (long long)orig[(size_t)v], pubs[(size_t)v]);
        std::fclose(f);
    }
    log.info("done: " + std::to_string(n) + " nodes, " + std::to_string(m) + " edges, " + std::to_string(total_edges) +
             " new edges in " + std::to_string(run_s) + " s");
    std::printf("E2E Time for num_cycles = %d with growth_rate = %g %% = %.3f seconds.\n", cycles, 100.0 * growth, run_s);
    pg_destroy(ctx);
    return 0;
}

}  // namespace
