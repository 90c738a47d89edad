// case_parser.cpp -- reads an OpenFOAM dsmcFoam+ case directory into a
// dsmc_case_spec: the dictionary subset the path uses and an axis-aligned,
// uniformly graded blockMeshDict.
//
// Dictionaries and keys (paths inside hystrath/hyStrath):
//   constant/dsmcProperties   nEquivalentParticles, BinaryCollisionModel and
//                             <Model>Coeffs (BinaryCollisionModel.C:59-90,
//                             VariableHardSphere.C:52-63,
//                             LarsenBorgnakkeVariableHardSphere.C:45-99),
//                             collisionPartnerSelectionModel
//                             (collisionPartnerSelection.C:64-97), typeIdList,
//                             moleculeProperties (dsmcParcelI.H:37-200), seedNumber
//   system/controlDict        deltaT
//   system/boundariesDict     dsmcPatchBoundaries (dsmcPatchBoundary.C:130-165),
//                             dsmcGeneralBoundaries (dsmcFreeStreamInflowPatch.C:393-475),
//                             dsmcCyclicBoundaries
//   system/fieldPropertiesDict dsmcVolFieldsProperties (dsmcVolFields.C:1030-1049)
//   system/dsmcInitialiseDict dsmcMeshFill configuration (dsmcMeshFill.C:68-110)
//   system/blockMeshDict      convertToMeters, vertices, blocks, patches/boundary
// Unknown model names are rejected with the list of valid names, as the
// reference's runtime-selection tables do.

#include <algorithm>
#include <array>
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <map>
#include <memory>
#include <set>
#include <sstream>
#include <string>
#include <vector>

#include "hystrath_gb300.h"

namespace dsmc {
void set_global_error(const std::string& msg);   // dsmc_api.cu
bool foam_cell_order(const std::string& dir, std::vector<long long>& order, std::string& err);
bool foam_read_scalar_field(const std::string& path, std::vector<double>& out, std::string& err);
}

namespace {

thread_local std::string g_perr;
thread_local std::vector<int> g_facePatch[6];

// ------------------------------------------------------------------ tokens
struct Tok {
    enum Kind { WORD, PUNCT, STRING, END } kind;
    std::string s;
};

class Lexer {
  public:
    explicit Lexer(const std::string& t) : t_(t) {}
    Tok next() {
        skip();
        if (p_ >= t_.size()) return {Tok::END, ""};
        const char c = t_[p_];
        if (c == '{' || c == '}' || c == '(' || c == ')' || c == ';' || c == '[' || c == ']') {
            ++p_;
            return {Tok::PUNCT, std::string(1, c)};
        }
        if (c == '"') {
            const size_t e = t_.find('"', p_ + 1);
            const std::string s = t_.substr(p_ + 1, e == std::string::npos ? std::string::npos : e - p_ - 1);
            p_ = (e == std::string::npos) ? t_.size() : e + 1;
            return {Tok::STRING, s};
        }
        const size_t b = p_;
        while (p_ < t_.size() && !std::isspace((unsigned char)t_[p_]) && !std::strchr("{}();[]\"", t_[p_])) {
            if (t_[p_] == '/' && p_ + 1 < t_.size() && (t_[p_ + 1] == '/' || t_[p_ + 1] == '*')) break;
            ++p_;
        }
        return {Tok::WORD, t_.substr(b, p_ - b)};
    }

  private:
    void skip() {
        for (;;) {
            while (p_ < t_.size() && std::isspace((unsigned char)t_[p_])) ++p_;
            if (p_ + 1 < t_.size() && t_[p_] == '/' && t_[p_ + 1] == '/') {
                while (p_ < t_.size() && t_[p_] != '\n') ++p_;
                continue;
            }
            if (p_ + 1 < t_.size() && t_[p_] == '/' && t_[p_ + 1] == '*') {
                const size_t e = t_.find("*/", p_ + 2);
                p_ = (e == std::string::npos) ? t_.size() : e + 2;
                continue;
            }
            break;
        }
    }
    const std::string& t_;
    size_t p_ = 0;
};

// ------------------------------------------------------------------ tree
struct Node {
    enum Kind { VALUE, LIST, DICT } kind = VALUE;
    std::vector<std::string> words;                          // VALUE
    std::vector<std::shared_ptr<Node>> items;                // LIST
    std::vector<std::string> itemNames;                      // LIST: name of a named dict item or ""
    std::vector<std::shared_ptr<Node>> more;                 // LIST: the value's later lists ("box (a) (b)")
    std::vector<std::pair<std::string, std::shared_ptr<Node>>> entries;  // DICT

    const Node* find(const std::string& k) const {
        for (auto& e : entries)
            if (e.first == k) return e.second.get();
        return nullptr;
    }
};

class Parser {
  public:
    explicit Parser(const std::string& text) : lex_(text) { cur_ = lex_.next(); }

    std::shared_ptr<Node> parseDict(bool top) {
        auto d = std::make_shared<Node>();
        d->kind = Node::DICT;
        for (;;) {
            if (cur_.kind == Tok::END) {
                if (!top) throw std::runtime_error("unexpected end of file inside a dictionary");
                return d;
            }
            if (cur_.kind == Tok::PUNCT && cur_.s == "}") {
                if (top) throw std::runtime_error("unbalanced '}'");
                advance();
                return d;
            }
            if (cur_.kind == Tok::PUNCT && cur_.s == ";") { advance(); continue; }
            if (cur_.kind != Tok::WORD && cur_.kind != Tok::STRING)
                throw std::runtime_error("expected a keyword, found '" + cur_.s + "'");
            const std::string key = cur_.s;
            advance();
            if (cur_.kind == Tok::PUNCT && cur_.s == "{") {
                advance();
                d->entries.emplace_back(key, parseDict(false));
            } else {
                d->entries.emplace_back(key, parseValue());
            }
        }
    }

  private:
    void advance() { cur_ = lex_.next(); }

    // Words and lists up to ';'.  As in OpenFOAM, an entry runs to the next
    // ';' (blockMeshDict files often omit it after "patches ( ... )", which
    // then swallows "mergePatchPairs ( )"); the entry's value is its first list.
    std::shared_ptr<Node> parseValue() {
        std::shared_ptr<Node> v = std::make_shared<Node>();
        v->kind = Node::VALUE;
        std::shared_ptr<Node> list;
        for (;;) {
            if (cur_.kind == Tok::END) throw std::runtime_error("missing ';'");
            if (cur_.kind == Tok::PUNCT && cur_.s == ";") { advance(); break; }
            if (cur_.kind == Tok::PUNCT && cur_.s == "(") {
                advance();
                auto l = parseList();
                if (!list) list = l;
                else list->more.push_back(l);
                continue;
            }
            if (list && cur_.kind == Tok::WORD) {   // words after the first list
                advance();
                continue;
            }
            if (cur_.kind == Tok::PUNCT && cur_.s == "[") {   // dimensions: skip
                while (!(cur_.kind == Tok::PUNCT && cur_.s == "]") && cur_.kind != Tok::END) advance();
                advance();
                continue;
            }
            if (cur_.kind == Tok::PUNCT && cur_.s == "}") throw std::runtime_error("missing ';' before '}'");
            v->words.push_back(cur_.s);
            advance();
        }
        if (list) {
            // "hex (0 1 2 ...)" style values keep their leading words
            list->words = v->words;
            return list;
        }
        return v;
    }

    std::shared_ptr<Node> parseList() {
        auto l = std::make_shared<Node>();
        l->kind = Node::LIST;
        for (;;) {
            if (cur_.kind == Tok::END) throw std::runtime_error("unterminated list");
            if (cur_.kind == Tok::PUNCT && cur_.s == ")") { advance(); return l; }
            if (cur_.kind == Tok::PUNCT && cur_.s == "(") {
                advance();
                l->items.push_back(parseList());
                l->itemNames.emplace_back();
                continue;
            }
            if (cur_.kind == Tok::PUNCT && cur_.s == "{") {   // anonymous dict item
                advance();
                l->items.push_back(parseDict(false));
                l->itemNames.emplace_back();
                continue;
            }
            if (cur_.kind == Tok::PUNCT && cur_.s == ";") { advance(); continue; }
            const std::string w = cur_.s;
            advance();
            if (cur_.kind == Tok::PUNCT && cur_.s == "{") {    // named dict item
                advance();
                l->items.push_back(parseDict(false));
                l->itemNames.push_back(w);
                continue;
            }
            auto v = std::make_shared<Node>();
            v->kind = Node::VALUE;
            v->words.push_back(w);
            l->items.push_back(v);
            l->itemNames.emplace_back();
        }
    }

    Lexer lex_;
    Tok cur_;
};

std::shared_ptr<Node> readDict(const std::string& path) {
    std::ifstream f(path);
    if (!f) throw std::runtime_error("cannot open " + path);
    std::stringstream ss;
    ss << f.rdbuf();
    const std::string text = ss.str();
    try {
        Parser p(text);
        return p.parseDict(true);
    } catch (const std::exception& e) {
        throw std::runtime_error(path + ": " + e.what());
    }
}

struct ParseError : std::runtime_error {
    int code;
    ParseError(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

double toNum(const std::string& w, const std::string& what) {
    char* end = nullptr;
    const double v = std::strtod(w.c_str(), &end);
    if (end == w.c_str() || *end) throw ParseError(DSMC_ERR_PARSE, what + ": '" + w + "' is not a number");
    return v;
}

const Node& need(const Node* d, const std::string& k, const std::string& where) {
    const Node* n = d ? d->find(k) : nullptr;
    if (!n) throw ParseError(DSMC_ERR_PARSE, "keyword " + k + " is undefined in " + where);
    return *n;
}

double scalar(const Node* d, const std::string& k, const std::string& where) {
    const Node& n = need(d, k, where);
    if (n.kind != Node::VALUE || n.words.size() != 1) throw ParseError(DSMC_ERR_PARSE, k + " in " + where + " is not a scalar");
    return toNum(n.words[0], k);
}

double scalarOr(const Node* d, const std::string& k, double def) {
    const Node* n = d ? d->find(k) : nullptr;
    if (!n || n->kind != Node::VALUE || n->words.size() != 1) return def;
    return toNum(n->words[0], k);
}

std::string word(const Node* d, const std::string& k, const std::string& where) {
    const Node& n = need(d, k, where);
    if (n.kind != Node::VALUE || n.words.size() != 1) throw ParseError(DSMC_ERR_PARSE, k + " in " + where + " is not a word");
    return n.words[0];
}

std::string wordOr(const Node* d, const std::string& k, const std::string& def) {
    const Node* n = d ? d->find(k) : nullptr;
    if (!n || n->kind != Node::VALUE || n->words.size() != 1) return def;
    return n->words[0];
}

std::vector<double> numList(const Node& n, const std::string& what) {
    std::vector<double> v;
    if (n.kind == Node::LIST) {
        for (auto& it : n.items) {
            if (it->kind != Node::VALUE || it->words.size() != 1) throw ParseError(DSMC_ERR_PARSE, what + ": nested list");
            v.push_back(toNum(it->words[0], what));
        }
    } else if (n.kind == Node::VALUE) {
        for (auto& w : n.words) v.push_back(toNum(w, what));
    }
    return v;
}

std::vector<std::string> wordList(const Node& n) {
    std::vector<std::string> v;
    if (n.kind == Node::LIST)
        for (auto& it : n.items)
            if (it->kind == Node::VALUE) v.insert(v.end(), it->words.begin(), it->words.end());
    return v;
}

bool boolOr(const Node* d, const std::string& k, bool def) {
    const std::string w = wordOr(d, k, "");
    if (w.empty()) return def;
    return w == "on" || w == "yes" || w == "true" || w == "1";
}

void copyName(char* dst, const std::string& s) {
    std::snprintf(dst, DSMC_NAME_LEN, "%s", s.c_str());
}

std::string fileIn(const std::string& dir, const char* a, const char* b = nullptr) {
    std::string p = dir + "/" + a;
    std::ifstream f(p);
    if (f || !b) return p;
    return dir + "/" + b;
}

// ------------------------------------------------------------------ mesh
// A hex block of blockMesh on the axis-aligned grid: its bounds, its cells
// along each global axis, the global axis and direction of each of its local
// directions (v0->v1, v0->v3, v0->v4) and its node coordinates along each
// global axis, ascending.
struct Block {
    double lo[3], hi[3];
    int n[3];
    int ax[3], dir[3];
    int cnt[3];                   // cells along the local directions
    std::vector<double> nodes[3];
};

// blockMesh's division of an edge of expansion ratio r into n cells
// (lineDivide): the widths grow geometrically, last / first = r.
std::vector<double> edge_division(int n, double r) {
    std::vector<double> lam((size_t)n + 1);
    if (n == 1 || std::fabs(r - 1.0) < 1e-12) {
        for (int i = 0; i <= n; ++i) lam[i] = (double)i / n;
    } else {
        const double q = std::pow(r, 1.0 / (n - 1));
        for (int i = 0; i <= n; ++i) lam[i] = (1.0 - std::pow(q, i)) / (1.0 - std::pow(q, n));
    }
    lam[0] = 0.0;
    lam[n] = 1.0;
    return lam;
}

std::vector<Block> parse_blocks(const Node& bn, const std::vector<std::array<double, 3>>& V) {
    std::vector<Block> blocks;
    for (size_t i = 0; i < bn.items.size(); ++i) {
        const Node& it = *bn.items[i];
        if (!(it.kind == Node::VALUE && !it.words.empty() && it.words[0] == "hex")) continue;
        // hex (v0..v7) [zoneName] (n1 n2 n3) simpleGrading (g1 g2 g3) | edgeGrading (12)
        if (i + 3 >= bn.items.size()) throw ParseError(DSMC_ERR_PARSE, "incomplete hex block");
        auto ids = numList(*bn.items[i + 1], "hex vertices");
        size_t ci = i + 2;
        if (bn.items[ci]->kind == Node::VALUE) ++ci;   // cell zone name
        if (ci + 1 >= bn.items.size()) throw ParseError(DSMC_ERR_PARSE, "incomplete hex block");
        auto cnt = numList(*bn.items[ci], "hex cell counts");
        if (ids.size() != 8 || cnt.size() != 3) throw ParseError(DSMC_ERR_PARSE, "malformed hex block");
        const Node& gw = *bn.items[ci + 1];
        size_t gi = ci;
        double g[3] = {1.0, 1.0, 1.0};
        if (gw.kind == Node::VALUE && !gw.words.empty() &&
            (gw.words[0] == "simpleGrading" || gw.words[0] == "edgeGrading")) {
            if (ci + 2 >= bn.items.size()) throw ParseError(DSMC_ERR_PARSE, "grading without values");
            const Node& gl = *bn.items[ci + 2];
            for (auto& e : gl.items)
                if (e->kind != Node::VALUE)
                    throw ParseError(DSMC_ERR_INVALID, "multi-section grading is not supported on this path");
            auto gv = numList(gl, "grading");
            if (gw.words[0] == "simpleGrading") {
                if (gv.size() != 3) throw ParseError(DSMC_ERR_PARSE, "simpleGrading needs 3 ratios");
                for (int l = 0; l < 3; ++l) g[l] = gv[l];
            } else {
                if (gv.size() != 12) throw ParseError(DSMC_ERR_PARSE, "edgeGrading needs 12 ratios");
                for (int l = 0; l < 3; ++l) {
                    for (int e = 1; e < 4; ++e)
                        if (std::fabs(gv[4 * l + e] - gv[4 * l]) > 1e-12 * std::fabs(gv[4 * l]))
                            throw ParseError(DSMC_ERR_INVALID, "edgeGrading with unequal parallel edges is not rectilinear");
                    g[l] = gv[4 * l];
                }
            }
            gi = ci + 2;
        }
        Block b{};
        for (int a = 0; a < 3; ++a) { b.lo[a] = 1e300; b.hi[a] = -1e300; }
        for (double id : ids) {
            const auto& p = V.at((size_t)id);
            for (int a = 0; a < 3; ++a) {
                b.lo[a] = std::min(b.lo[a], p[a]);
                b.hi[a] = std::max(b.hi[a], p[a]);
            }
        }
        for (double id : ids) {
            const auto& p = V.at((size_t)id);
            for (int a = 0; a < 3; ++a) {
                const double tol = 1e-9 * (b.hi[a] - b.lo[a] + 1e-300);
                if (std::fabs(p[a] - b.lo[a]) > tol && std::fabs(p[a] - b.hi[a]) > tol)
                    throw ParseError(DSMC_ERR_INVALID, "hex block is not an axis-aligned box");
            }
        }
        // local directions: v0 -> v1, v0 -> v3, v0 -> v4
        const auto& v0 = V.at((size_t)ids[0]);
        const int other[3] = {1, 3, 4};
        int used = 0;
        for (int l = 0; l < 3; ++l) {
            const auto& v = V.at((size_t)ids[other[l]]);
            int axis = -1;
            for (int a = 0; a < 3; ++a) {
                const double tol = 1e-9 * (b.hi[a] - b.lo[a] + 1e-300);
                if (std::fabs(v[a] - v0[a]) > tol) {
                    if (axis >= 0) throw ParseError(DSMC_ERR_INVALID, "hex block edge is not axis-aligned");
                    axis = a;
                }
            }
            if (axis < 0 || (used >> axis) & 1) throw ParseError(DSMC_ERR_INVALID, "degenerate hex block");
            used |= 1 << axis;
            b.ax[l] = axis;
            b.dir[l] = v[axis] > v0[axis] ? 1 : -1;
            b.cnt[l] = (int)cnt[l];
            if (b.cnt[l] < 1) throw ParseError(DSMC_ERR_INVALID, "hex block with no cells");
            b.n[axis] = b.cnt[l];
            const double L = b.hi[axis] - b.lo[axis];
            const std::vector<double> lam = edge_division(b.cnt[l], g[l]);
            std::vector<double>& nd = b.nodes[axis];
            nd.resize(lam.size());
            for (size_t k = 0; k < lam.size(); ++k)
                nd[b.dir[l] > 0 ? k : lam.size() - 1 - k] = b.dir[l] > 0 ? b.lo[axis] + L * lam[k]
                                                                       : b.hi[axis] - L * lam[k];
            nd.front() = b.lo[axis];
            nd.back() = b.hi[axis];
        }
        blocks.push_back(b);
        i = gi;
    }
    return blocks;
}

// The global nodes of every axis from the blocks' nodes; blocks must meet
// node to node (a rectilinear grid).  Returns true when the axis is uniform.
bool merge_axis_nodes(const std::vector<Block>& blocks, int a, std::vector<double>& out) {
    double lo = 1e300, hi = -1e300;
    for (auto& b : blocks) { lo = std::min(lo, b.lo[a]); hi = std::max(hi, b.hi[a]); }
    const double tol = 1e-9 * (hi - lo);
    std::vector<double> all;
    for (auto& b : blocks) all.insert(all.end(), b.nodes[a].begin(), b.nodes[a].end());
    std::sort(all.begin(), all.end());
    out.clear();
    for (double x : all)
        if (out.empty() || x - out.back() > tol) out.push_back(x);
    for (auto& b : blocks) {
        size_t k = 0;
        while (k < out.size() && out[k] < b.lo[a] - tol) ++k;
        for (double x : b.nodes[a]) {
            if (k >= out.size() || std::fabs(out[k] - x) > tol)
                throw ParseError(DSMC_ERR_INVALID, "blocks whose cells do not meet face to face are not supported");
            ++k;
        }
    }
    const double w0 = (out.back() - out.front()) / (double)(out.size() - 1);
    bool uniform = true;
    for (size_t k = 1; k < out.size(); ++k)
        if (std::fabs((out[k] - out[k - 1]) - w0) > 1e-9 * w0) uniform = false;
    return uniform;
}

thread_local std::vector<double> g_nodes[3];

void readMesh(const std::string& dir, dsmc_case_spec* s, std::map<std::string, int>& patchIds,
              std::vector<std::string>& patchTypes) {
    const std::string path = fileIn(dir, "system/blockMeshDict", "constant/polyMesh/blockMeshDict");
    auto bm = readDict(path);
    const double scale = scalarOr(bm.get(), "convertToMeters", scalarOr(bm.get(), "scale", 1.0));
    const Node& vn = need(bm.get(), "vertices", path);
    std::vector<std::array<double, 3>> V;
    for (auto& it : vn.items) {
        auto c = numList(*it, "vertex");
        if (c.size() != 3) throw ParseError(DSMC_ERR_PARSE, "vertex with " + std::to_string(c.size()) + " coordinates");
        V.push_back({c[0] * scale, c[1] * scale, c[2] * scale});
    }
    const Node& bn = need(bm.get(), "blocks", path);
    std::vector<Block> blocks = parse_blocks(bn, V);
    if (blocks.empty()) throw ParseError(DSMC_ERR_PARSE, path + ": no hex blocks");
    double dx[3], lo[3], hi[3];
    for (int a = 0; a < 3; ++a) {
        std::vector<double>& nd = g_nodes[a];
        const bool uniform = merge_axis_nodes(blocks, a, nd);
        lo[a] = nd.front();
        hi[a] = nd.back();
        s->n_cells[a] = (int)nd.size() - 1;
        s->origin[a] = lo[a];
        s->cell_size[a] = (hi[a] - lo[a]) / s->n_cells[a];
        s->node_coords[a] = uniform ? nullptr : nd.data();
        dx[a] = s->cell_size[a];
        for (size_t k = 1; k < nd.size(); ++k) dx[a] = std::min(dx[a], nd[k] - nd[k - 1]);
    }
    const int nx = s->n_cells[0], ny = s->n_cells[1], nz = s->n_cells[2];
    // index of the global node at coordinate x
    auto idx = [&](double x, int a) {
        const std::vector<double>& nd = g_nodes[a];
        const size_t k = (size_t)(std::lower_bound(nd.begin(), nd.end(), x - 1e-9 * (hi[a] - lo[a])) - nd.begin());
        if (k >= nd.size() || std::fabs(nd[k] - x) > 1e-9 * (hi[a] - lo[a]))
            throw ParseError(DSMC_ERR_INVALID, "a block or face corner is not on a mesh node");
        return (int)k;
    };
    std::vector<unsigned char> covered((size_t)nx * ny * nz, 0);
    for (auto& b : blocks) {
        int l[3], h[3];
        for (int a = 0; a < 3; ++a) { l[a] = idx(b.lo[a], a); h[a] = idx(b.hi[a], a); }
        for (int k = l[2]; k < h[2]; ++k)
            for (int j = l[1]; j < h[1]; ++j)
                for (int i = l[0]; i < h[0]; ++i) covered[i + (size_t)nx * (j + (size_t)ny * k)] = 1;
    }
    // uncovered cells become solid boxes (greedy decomposition)
    s->n_obstacles = 0;
    std::vector<unsigned char> todo(covered.size());
    for (size_t c = 0; c < covered.size(); ++c) todo[c] = !covered[c];
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                if (!todo[i + (size_t)nx * (j + (size_t)ny * k)]) continue;
                int i1 = i, j1 = j, k1 = k;
                while (i1 + 1 < nx && todo[(i1 + 1) + (size_t)nx * (j + (size_t)ny * k)]) ++i1;
                auto rowOk = [&](int jj, int kk) {
                    for (int ii = i; ii <= i1; ++ii)
                        if (!todo[ii + (size_t)nx * (jj + (size_t)ny * kk)]) return false;
                    return true;
                };
                while (j1 + 1 < ny && rowOk(j1 + 1, k)) ++j1;
                auto planeOk = [&](int kk) {
                    for (int jj = j; jj <= j1; ++jj)
                        if (!rowOk(jj, kk)) return false;
                    return true;
                };
                while (k1 + 1 < nz && planeOk(k1 + 1)) ++k1;
                if (s->n_obstacles >= DSMC_MAX_OBSTACLES)
                    throw ParseError(DSMC_ERR_INVALID, "the mesh leaves more than 8 solid boxes uncovered");
                dsmc_obstacle& ob = s->obstacles[s->n_obstacles++];
                ob.lo[0] = i; ob.lo[1] = j; ob.lo[2] = k;
                ob.hi[0] = i1 + 1; ob.hi[1] = j1 + 1; ob.hi[2] = k1 + 1;
                for (int q = 0; q < 6; ++q) ob.patch[q] = -1;
                for (int kk = k; kk <= k1; ++kk)
                    for (int jj = j; jj <= j1; ++jj)
                        for (int ii = i; ii <= i1; ++ii) todo[ii + (size_t)nx * (jj + (size_t)ny * kk)] = 0;
            }

    // patches: old "patches ( type name ( faces ) ... )" or new "boundary ( name { type; faces; } )"
    struct PatchFaces { std::string name, type; std::vector<std::vector<double>> faces; };
    std::vector<PatchFaces> pf;
    if (const Node* pn = bm->find("boundary")) {
        for (size_t i = 0; i < pn->items.size(); ++i) {
            if (pn->items[i]->kind != Node::DICT) continue;
            PatchFaces p;
            p.name = pn->itemNames[i];
            p.type = word(pn->items[i].get(), "type", "boundary " + p.name);
            const Node& f = need(pn->items[i].get(), "faces", "boundary " + p.name);
            for (auto& it : f.items) p.faces.push_back(numList(*it, "face"));
            pf.push_back(p);
        }
    } else if (const Node* pn = bm->find("patches")) {
        // groups of three items: type, name, list of faces
        for (size_t i = 0; i + 2 < pn->items.size(); i += 3) {
            const Node& t = *pn->items[i];
            const Node& nm = *pn->items[i + 1];
            const Node& fl = *pn->items[i + 2];
            if (t.kind != Node::VALUE || nm.kind != Node::VALUE || fl.kind != Node::LIST)
                throw ParseError(DSMC_ERR_PARSE, path + ": malformed patches entry");
            PatchFaces p;
            p.type = t.words.empty() ? "" : t.words[0];
            p.name = nm.words.empty() ? "" : nm.words[0];
            for (auto& it : fl.items) p.faces.push_back(numList(*it, "face"));
            pf.push_back(p);
        }
    } else {
        throw ParseError(DSMC_ERR_PARSE, path + ": neither boundary nor patches");
    }
    for (int q = 0; q < 6; ++q) {
        const int a = q / 2, b = (a == 0) ? 1 : 0, c = (a == 2) ? 1 : 2;
        g_facePatch[q].assign((size_t)s->n_cells[b] * s->n_cells[c], -1);
    }
    for (auto& p : pf) {
        int type;
        if (p.type == "wall") type = DSMC_PATCH_WALL;
        else if (p.type == "patch") type = DSMC_PATCH_PATCH;
        else if (p.type == "symmetry" || p.type == "symmetryPlane") type = DSMC_PATCH_SYMMETRY;
        else if (p.type == "cyclic") type = DSMC_PATCH_CYCLIC;
        else if (p.type == "empty") type = DSMC_PATCH_EMPTY;
        else
            throw ParseError(DSMC_ERR_INVALID, "patch " + p.name + ": unsupported patch type " + p.type +
                                                   "; valid: wall patch symmetry symmetryPlane cyclic empty");
        if (s->n_patches >= DSMC_MAX_PATCHES) throw ParseError(DSMC_ERR_INVALID, "more than 16 patches");
        const int pid = s->n_patches++;
        copyName(s->patches[pid].name, p.name);
        s->patches[pid].type = type;
        patchIds[p.name] = pid;
        patchTypes.push_back(p.type);
        for (auto& f : p.faces) {
            if (f.size() != 4) throw ParseError(DSMC_ERR_PARSE, "patch " + p.name + ": face without 4 vertices");
            double flo[3] = {1e300, 1e300, 1e300}, fhi[3] = {-1e300, -1e300, -1e300};
            for (double id : f) {
                const auto& v = V.at((size_t)id);
                for (int a = 0; a < 3; ++a) { flo[a] = std::min(flo[a], v[a]); fhi[a] = std::max(fhi[a], v[a]); }
            }
            int axis = -1;
            for (int a = 0; a < 3; ++a)
                if (fhi[a] - flo[a] <= 1e-9 * dx[a]) axis = a;
            if (axis < 0) throw ParseError(DSMC_ERR_INVALID, "patch " + p.name + ": face is not axis-aligned");
            const int b = (axis == 0) ? 1 : 0, c = (axis == 2) ? 1 : 2;
            const int pl = idx(flo[axis], axis);
            const int b0 = idx(flo[b], b), b1 = idx(fhi[b], b), c0 = idx(flo[c], c), c1 = idx(fhi[c], c);
            int side = -1;
            if (pl == 0) side = 2 * axis;
            else if (pl == s->n_cells[axis]) side = 2 * axis + 1;
            if (side >= 0) {
                for (int cc = c0; cc < c1; ++cc)
                    for (int bb = b0; bb < b1; ++bb) g_facePatch[side][bb + (size_t)s->n_cells[b] * cc] = pid;
            } else {
                // a face on the surface of a solid box
                bool placed = false;
                for (int o = 0; o < s->n_obstacles && !placed; ++o) {
                    dsmc_obstacle& ob = s->obstacles[o];
                    if (b0 < ob.lo[b] || b1 > ob.hi[b] || c0 < ob.lo[c] || c1 > ob.hi[c]) continue;
                    if (pl == ob.lo[axis]) { ob.patch[2 * axis] = pid; placed = true; }
                    else if (pl == ob.hi[axis]) { ob.patch[2 * axis + 1] = pid; placed = true; }
                }
                if (!placed) throw ParseError(DSMC_ERR_INVALID, "patch " + p.name + ": face is neither on the domain nor on a solid box");
            }
        }
    }
    static const char* sideName[6] = {"-x", "+x", "-y", "+y", "-z", "+z"};
    int defaultPatch = -1;
    for (int q = 0; q < 6; ++q) {
        const int a = q / 2, b = (a == 0) ? 1 : 0, c = (a == 2) ? 1 : 2;
        for (size_t f = 0; f < g_facePatch[q].size(); ++f) {
            if (g_facePatch[q][f] >= 0) continue;
            // a side face whose cell is solid belongs to no mesh cell and is never hit
            int ci[3];
            ci[a] = (q & 1) ? s->n_cells[a] - 1 : 0;
            ci[b] = (int)(f % s->n_cells[b]);
            ci[c] = (int)(f / s->n_cells[b]);
            if (!covered[ci[0] + (size_t)nx * (ci[1] + (size_t)ny * ci[2])]) {
                g_facePatch[q][f] = 0;
                continue;
            }
            // blockMesh puts faces listed in no patch into its default patch
            // (defaultPatch { name defaultFaces; type empty; })
            if (defaultPatch < 0) {
                if (s->n_patches >= DSMC_MAX_PATCHES) throw ParseError(DSMC_ERR_INVALID, "more than 16 patches");
                defaultPatch = s->n_patches++;
                std::string dn = "defaultFaces", dt = "empty";
                if (const Node* dp = bm->find("defaultPatch")) {
                    dn = wordOr(dp, "name", dn);
                    dt = wordOr(dp, "type", dt);
                }
                int type;
                if (dt == "empty") type = DSMC_PATCH_EMPTY;
                else if (dt == "wall") type = DSMC_PATCH_WALL;
                else if (dt == "patch") type = DSMC_PATCH_PATCH;
                else if (dt == "symmetry" || dt == "symmetryPlane") type = DSMC_PATCH_SYMMETRY;
                else throw ParseError(DSMC_ERR_INVALID, "defaultPatch " + dn + ": unsupported patch type " + dt);
                copyName(s->patches[defaultPatch].name, dn);
                s->patches[defaultPatch].type = type;
                patchIds[dn] = defaultPatch;
                patchTypes.push_back(dt);
            }
            (void)sideName;
            g_facePatch[q][f] = defaultPatch;
        }
        s->face_patch[q] = g_facePatch[q].data();
        s->side_patch[q] = g_facePatch[q].empty() ? 0 : g_facePatch[q][0];
    }
    for (int o = 0; o < s->n_obstacles; ++o)
        for (int q = 0; q < 6; ++q) {
            dsmc_obstacle& ob = s->obstacles[o];
            const int a = q / 2;
            // faces of a solid box that touch the domain side are never hit
            const bool onSide = (q & 1) ? ob.hi[a] == s->n_cells[a] : ob.lo[a] == 0;
            if (ob.patch[q] < 0 && !onSide)
                throw ParseError(DSMC_ERR_INVALID, "a solid box face has no patch");
            if (ob.patch[q] < 0) ob.patch[q] = 0;
        }
}

void readCase(const std::string& dir, dsmc_case_spec* s) {
    dsmc_spec_defaults(s);
    std::map<std::string, int> patchIds;
    std::vector<std::string> patchTypes;
    readMesh(dir, s, patchIds, patchTypes);

    // constant/dsmcProperties
    const std::string dpPath = dir + "/constant/dsmcProperties";
    auto dp = readDict(dpPath);
    s->n_equivalent_particles = scalar(dp.get(), "nEquivalentParticles", dpPath);
    const std::string bcm = word(dp.get(), "BinaryCollisionModel", dpPath);
    if (bcm == "VariableHardSphere") s->binary_collision_model = DSMC_COLL_VHS;
    else if (bcm == "LarsenBorgnakkeVariableHardSphere") s->binary_collision_model = DSMC_COLL_LB_VHS;
    else if (bcm == "VariableSoftSphere") s->binary_collision_model = DSMC_COLL_VSS;
    else if (bcm == "LarsenBorgnakkeVariableSoftSphere") s->binary_collision_model = DSMC_COLL_LB_VSS;
    else
        throw ParseError(DSMC_ERR_UNKNOWN_MODEL, "Unknown BinaryCollisionModel type " + bcm +
                                                     ". Valid BinaryCollisionModel types are: 4(VariableHardSphere "
                                                     "LarsenBorgnakkeVariableHardSphere VariableSoftSphere "
                                                     "LarsenBorgnakkeVariableSoftSphere)");
    if (const Node* co = dp->find(bcm + "Coeffs")) {
        s->tref = scalarOr(co, "Tref", 273.0);
        s->zrot = scalarOr(co, "rotationalRelaxationCollisionNumber", 5.0);
        s->fixed_zv = scalarOr(co, "vibrationalRelaxationCollisionNumber", 0.0);
        const std::string f = wordOr(co, "inverseZvFormulation", "");
        s->inv_zv_formulation = (f == "pre-2008") ? 0 : (f == "2008") ? 1 : 2;
    }
    const std::string sel = word(dp.get(), "collisionPartnerSelectionModel", dpPath);
    if (sel == "noTimeCounter") s->partner_selection_model = DSMC_SEL_NTC;
    else if (sel == "simplifiedBernoulliTrials") s->partner_selection_model = DSMC_SEL_SBT;
    else
        throw ParseError(DSMC_ERR_UNKNOWN_MODEL, "Unknown collisionPartnerSelectionModel type " + sel +
                                                     ". Valid collisionPartnerSelectionModel types are: "
                                                     "2(noTimeCounter simplifiedBernoulliTrials)");
    s->seed = (unsigned long long)scalarOr(dp.get(), "seedNumber", 0.0);
    const std::vector<std::string> types = wordList(need(dp.get(), "typeIdList", dpPath));
    if (types.empty() || types.size() > DSMC_MAX_SPECIES)
        throw ParseError(DSMC_ERR_INVALID, "typeIdList must hold 1..8 species");
    const Node& mp = need(dp.get(), "moleculeProperties", dpPath);
    s->n_species = (int)types.size();
    std::map<std::string, int> spId;
    for (size_t i = 0; i < types.size(); ++i) {
        const Node& m = need(&mp, types[i], "moleculeProperties");
        dsmc_species& q = s->species[i];
        copyName(q.name, types[i]);
        q.mass = scalar(&m, "mass", types[i]);
        q.diameter = scalar(&m, "diameter", types[i]);
        q.omega = scalar(&m, "omega", types[i]);
        q.alpha = scalarOr(&m, "alpha", 1.0);
        q.rotational_dof = scalarOr(&m, "rotationalDegreesOfFreedom", 0.0);
        q.n_vib_modes = (int)scalarOr(&m, "nVibrationalModes", 0.0);
        if (q.n_vib_modes > 1)
            throw ParseError(DSMC_ERR_INVALID, types[i] + ": more than one vibrational mode is not supported on this path");
        if (q.n_vib_modes == 1) {
            q.theta_v = numList(need(&m, "characteristicVibrationalTemperature", types[i]), "thetaV").at(0);
            q.theta_d = scalarOr(&m, "dissociationTemperature", 0.0);
            q.zref = numList(need(&m, "Zref", types[i]), "Zref").at(0);
            q.tref_zv = numList(need(&m, "referenceTempForZref", types[i]), "TrefZv").at(0);
        }
        spId[types[i]] = (int)i;
    }

    // system/controlDict
    const std::string cdPath = dir + "/system/controlDict";
    auto cd = readDict(cdPath);
    s->delta_t = scalar(cd.get(), "deltaT", cdPath);
    // output times: writeControl timeStep (every writeInterval steps) or
    // runTime / adjustableRunTime (every writeInterval seconds)
    {
        const double wi = scalarOr(cd.get(), "writeInterval", 0.0);
        const std::string wc = wordOr(cd.get(), "writeControl", "timeStep");
        if (wi > 0) {
            const double steps = (wc == "timeStep") ? wi : wi / s->delta_t;
            s->write_interval_steps = (long long)std::llround(steps);
            if (s->write_interval_steps < 1) s->write_interval_steps = 1;
        }
    }

    // system/boundariesDict
    const std::string bdPath = dir + "/system/boundariesDict";
    auto bd = readDict(bdPath);
    if (const Node* pbs = bd->find("dsmcPatchBoundaries")) {
        for (auto& it : pbs->items) {
            if (it->kind != Node::DICT) continue;
            const Node* props = &need(it.get(), "patchBoundaryProperties", "dsmcPatchBoundaries");
            const std::string pname = word(props, "patchName", "patchBoundaryProperties");
            auto pi = patchIds.find(pname);
            if (pi == patchIds.end()) throw ParseError(DSMC_ERR_INVALID, "Cannot find patch: " + pname + " in " + bdPath);
            const std::string model = word(it.get(), "boundaryModel", "dsmcPatchBoundaries");
            dsmc_patch& pt = s->patches[pi->second];
            const Node* mprops = it->find(model + "Properties");
            if (model == "dsmcSpecularWallPatch") pt.model = DSMC_BC_SPECULAR;
            else if (model == "dsmcDeletionPatch") pt.model = DSMC_BC_DELETION;
            else if (model == "dsmcDiffuseWallPatch") {
                pt.model = DSMC_BC_DIFFUSE;
                pt.wall_temperature = scalar(mprops, "temperature", model + "Properties");
                if (const Node* v = mprops ? mprops->find("velocity") : nullptr) {
                    auto u = numList(*v, "velocity");
                    for (int a = 0; a < 3 && a < (int)u.size(); ++a) pt.wall_velocity[a] = u[a];
                }
            } else {
                throw ParseError(DSMC_ERR_UNKNOWN_MODEL, "Unknown dsmcPatchBoundary type " + model +
                                                             ". Valid dsmcPatchBoundary types on this path are: "
                                                             "3(dsmcSpecularWallPatch dsmcDiffuseWallPatch dsmcDeletionPatch)");
            }
        }
    }
    if (const Node* gbs = bd->find("dsmcGeneralBoundaries")) {
        for (auto& it : gbs->items) {
            if (it->kind != Node::DICT) continue;
            const Node* props = &need(it.get(), "generalBoundaryProperties", "dsmcGeneralBoundaries");
            const std::string pname = word(props, "patchName", "generalBoundaryProperties");
            auto pi = patchIds.find(pname);
            if (pi == patchIds.end()) throw ParseError(DSMC_ERR_INVALID, "Cannot find patch: " + pname + " in " + bdPath);
            const std::string model = word(it.get(), "boundaryModel", "dsmcGeneralBoundaries");
            if (model != "dsmcFreeStreamInflowPatch")
                throw ParseError(DSMC_ERR_UNKNOWN_MODEL, "Unknown dsmcGeneralBoundary type " + model +
                                                             ". Valid dsmcGeneralBoundary types on this path are: "
                                                             "1(dsmcFreeStreamInflowPatch)");
            const Node* mprops = &need(it.get(), model + "Properties", "dsmcGeneralBoundaries");
            dsmc_patch& pt = s->patches[pi->second];
            pt.inflow = 1;
            const Node& nd = need(mprops, "numberDensities", model + "Properties");
            for (auto& e : nd.entries) {
                auto si = spId.find(e.first);
                if (si == spId.end()) throw ParseError(DSMC_ERR_INVALID, "inflow species " + e.first + " is not in typeIdList");
                pt.inflow_number_density[si->second] = numList(*e.second, "numberDensity").at(0);
            }
            pt.inflow_t_tra = scalar(mprops, "translationalTemperature", model + "Properties");
            pt.inflow_t_rot = scalarOr(mprops, "rotationalTemperature", pt.inflow_t_tra);
            pt.inflow_t_vib = scalarOr(mprops, "vibrationalTemperature", pt.inflow_t_tra);
            auto u = numList(need(mprops, "velocity", model + "Properties"), "velocity");
            for (int a = 0; a < 3 && a < (int)u.size(); ++a) pt.inflow_velocity[a] = u[a];
        }
    }
    for (int p = 0; p < s->n_patches; ++p) {
        const dsmc_patch& pt = s->patches[p];
        if ((pt.type == DSMC_PATCH_WALL || pt.type == DSMC_PATCH_PATCH) && pt.model == DSMC_BC_NONE)
            throw ParseError(DSMC_ERR_INVALID, std::string("patch ") + pt.name +
                                                   " has no dsmcPatchBoundaries model in " + bdPath);
    }

    // system/fieldPropertiesDict (optional)
    {
        std::ifstream probe(dir + "/system/fieldPropertiesDict");
        if (probe) {
            auto fp = readDict(dir + "/system/fieldPropertiesDict");
            if (const Node* fl = fp->find("dsmcFields")) {
                for (auto& it : fl->items) {
                    if (it->kind != Node::DICT) continue;
                    const std::string model = wordOr(it.get(), "fieldModel", "");
                    if (model != "dsmcVolFields") continue;
                    const Node* pr = it->find("dsmcVolFieldsProperties");
                    s->measure_mean_free_path = boolOr(pr, "measureMeanFreePath", false) ? 1 : 0;
                    s->mfp_tref = scalarOr(pr, "mfpReferenceTemperature", 273.0);
                    s->measure_errors = boolOr(pr, "measureErrors", false) ? 1 : 0;
                    s->measure_heat_flux_shear_stress = boolOr(pr, "measureHeatFluxShearStress", false) ? 1 : 0;
                    if (const Node* tp = it->find("timeProperties")) {
                        s->reset_at_output = boolOr(tp, "resetAtOutput", false) ? 1 : 0;
                        s->reset_at_output_until_time = scalarOr(tp, "resetAtOutputUntilTime", 0.0);
                    }
                }
            }
        }
    }

    // system/dsmcInitialiseDict
    const std::string idPath = dir + "/system/dsmcInitialiseDict";
    auto id = readDict(idPath);
    const Node& cfgs = need(id.get(), "configurations", idPath);
    bool filled = false;
    for (auto& it : cfgs.items) {
        if (it->kind != Node::DICT) continue;
        const std::string type = word(it.get(), "type", "configuration");
        if (type != "dsmcMeshFill")
            throw ParseError(DSMC_ERR_UNKNOWN_MODEL, "Unknown configuration type " + type +
                                                         ". Valid configuration types on this path are: 1(dsmcMeshFill)");
        const Node& nd = need(it.get(), "numberDensities", "dsmcMeshFill");
        for (auto& e : nd.entries) {
            auto si = spId.find(e.first);
            if (si == spId.end()) throw ParseError(DSMC_ERR_INVALID, "mesh-fill species " + e.first + " is not in typeIdList");
            s->init_number_density[si->second] = numList(*e.second, "numberDensity").at(0);
        }
        s->init_t_tra = scalar(it.get(), "translationalTemperature", "dsmcMeshFill");
        s->init_t_rot = scalar(it.get(), "rotationalTemperature", "dsmcMeshFill");
        s->init_t_vib = scalar(it.get(), "vibrationalTemperature", "dsmcMeshFill");
        auto u = numList(need(it.get(), "velocity", "dsmcMeshFill"), "velocity");
        for (int a = 0; a < 3 && a < (int)u.size(); ++a) s->init_velocity[a] = u[a];
        filled = true;
    }
    if (!filled) throw ParseError(DSMC_ERR_PARSE, idPath + ": no configuration");
}

}  // namespace

// OpenFOAM's cell order of the case's blockMesh (block by block in the
// blocks list, i fastest within a block) as Cartesian indices
// i + nx (j + ny k) of the merged uniform grid.
bool dsmc::foam_cell_order(const std::string& dir, std::vector<long long>& order, std::string& err) {
    try {
        dsmc_case_spec s{};
        std::map<std::string, int> patchIds;
        std::vector<std::string> patchTypes;
        readMesh(dir, &s, patchIds, patchTypes);
        const std::string path = fileIn(dir, "system/blockMeshDict", "constant/polyMesh/blockMeshDict");
        auto bm = readDict(path);
        const double scale = scalarOr(bm.get(), "convertToMeters", scalarOr(bm.get(), "scale", 1.0));
        const Node& vn = need(bm.get(), "vertices", path);
        std::vector<std::array<double, 3>> V;
        for (auto& it : vn.items) {
            auto c = numList(*it, "vertex");
            V.push_back({c[0] * scale, c[1] * scale, c[2] * scale});
        }
        const std::vector<Block> blocks = parse_blocks(need(bm.get(), "blocks", path), V);
        order.clear();
        for (const Block& b : blocks) {
            // first global cell of the block along each axis
            int o[3];
            for (int a = 0; a < 3; ++a) {
                const std::vector<double>& nd = g_nodes[a];
                const double tol = 1e-9 * (nd.back() - nd.front());
                o[a] = (int)(std::lower_bound(nd.begin(), nd.end(), b.lo[a] - tol) - nd.begin());
            }
            // blockMesh numbers a block's cells along its local directions,
            // the first fastest, each from the block's vertex 0
            int l3[3];
            for (l3[2] = 0; l3[2] < b.cnt[2]; ++l3[2])
                for (l3[1] = 0; l3[1] < b.cnt[1]; ++l3[1])
                    for (l3[0] = 0; l3[0] < b.cnt[0]; ++l3[0]) {
                        int g[3];
                        for (int l = 0; l < 3; ++l) {
                            const int a = b.ax[l];
                            g[a] = o[a] + (b.dir[l] > 0 ? l3[l] : b.cnt[l] - 1 - l3[l]);
                        }
                        order.push_back(g[0] + (long long)s.n_cells[0] * (g[1] + (long long)s.n_cells[1] * g[2]));
                    }
        }
        return true;
    } catch (const std::exception& e) {
        err = e.what();
        return false;
    }
}

extern "C" int dsmc_parse_case(const char* case_dir, dsmc_case_spec* spec) {
    try {
        readCase(case_dir, spec);
        return DSMC_OK;
    } catch (const ParseError& e) {
        g_perr = e.what();
        dsmc::set_global_error(g_perr);
        return e.code;
    } catch (const std::exception& e) {
        g_perr = e.what();
        dsmc::set_global_error(g_perr);
        return (g_perr.find("cannot open") != std::string::npos) ? DSMC_ERR_IO : DSMC_ERR_PARSE;
    }
}

extern "C" const char* dsmc_parse_last_error(void) { return g_perr.c_str(); }

// ------------------------------------------------------------------ lagrangian
// The parcel files of a dsmcFoam+ time directory, as dsmcParcelIO writes
// them (dsmcParcelIO.C:133-450): one IOField per file, "N (items)" or
// "N{uniform item}" after the FoamFile header.
namespace {

struct ListTokens {
    std::string text;
    std::vector<Tok> t;
    size_t i = 0;
    const Tok& peek() const { static const Tok end{Tok::END, ""}; return i < t.size() ? t[i] : end; }
    Tok take() { Tok k = peek(); ++i; return k; }
    void expect(const char* p, const std::string& where) {
        const Tok k = take();
        if (k.kind != Tok::PUNCT || k.s != p) throw ParseError(DSMC_ERR_PARSE, where + ": expected '" + p + "'");
    }
};

// Tokens of a field file after its FoamFile header; false when the file is absent.
bool field_tokens(const std::string& path, ListTokens& L) {
    std::ifstream f(path, std::ios::binary);
    if (!f) return false;
    std::stringstream ss;
    ss << f.rdbuf();
    L.text = ss.str();
    Lexer lx(L.text);
    for (Tok k = lx.next(); k.kind != Tok::END; k = lx.next()) L.t.push_back(k);
    if (L.peek().kind == Tok::WORD && L.peek().s == "FoamFile") {
        L.take();
        L.expect("{", path);
        int depth = 1;
        while (depth > 0 && L.peek().kind != Tok::END) {
            const Tok k = L.take();
            if (k.kind == Tok::PUNCT && k.s == "{") ++depth;
            if (k.kind == Tok::PUNCT && k.s == "}") --depth;
        }
    }
    return true;
}

double tok_num(const Tok& k, const std::string& where) {
    char* e = nullptr;
    const double v = std::strtod(k.s.c_str(), &e);
    if (k.kind != Tok::WORD || e == k.s.c_str() || *e) throw ParseError(DSMC_ERR_PARSE, where + ": expected a number");
    return v;
}

// Reads "N" then the items; item(L) parses one item at index k.  A uniform
// list "N{item}" repeats its item.
template <class F>
long long read_list(ListTokens& L, const std::string& where, F item) {
    const long long n = (long long)tok_num(L.take(), where);
    if (n < 0) throw ParseError(DSMC_ERR_PARSE, where + ": negative size");
    if (L.peek().kind == Tok::PUNCT && L.peek().s == "{") {
        L.take();
        const size_t at = L.i;
        for (long long k = 0; k < n; ++k) { L.i = at; item(k); }
        if (n == 0) item(-1);
        L.expect("}", where);
        return n;
    }
    L.expect("(", where);
    for (long long k = 0; k < n; ++k) item(k);
    L.expect(")", where);
    return n;
}

void read_vector(ListTokens& L, const std::string& where, double* v) {
    L.expect("(", where);
    for (int a = 0; a < 3; ++a) v[a] = tok_num(L.take(), where);
    if (!(L.peek().kind == Tok::PUNCT && L.peek().s == ")"))
        throw ParseError(DSMC_ERR_INVALID, where + ": barycentric positions (OpenFOAM 5 and later) are not supported; "
                                               "positions must be Cartesian (x y z) celli");
    L.expect(")", where);
}

struct ParcelArrays {
    long long n = -1;
    std::vector<double> pos, U, erot;
    std::vector<int> vib, species;
    std::vector<unsigned> id;
};

void read_parcel_files(const std::string& dir, ParcelArrays& P) {
    ListTokens L;
    const std::string pp = dir + "/positions";
    if (!field_tokens(pp, L)) throw ParseError(DSMC_ERR_IO, "cannot open " + pp);
    // (x y z) celli [tetFacei tetPti]: the cell labels are not needed, the
    // positions decide the cells
    const long long n = read_list(L, pp, [&](long long k) {
        double v[3];
        read_vector(L, pp, v);
        while (L.peek().kind == Tok::WORD) L.take();
        if (k < 0) return;
        if ((long long)P.pos.size() < 3 * (k + 1)) P.pos.resize(3 * (size_t)(k + 1));
        for (int a = 0; a < 3; ++a) P.pos[3 * (size_t)k + a] = v[a];
    });
    P.n = n;
    P.pos.resize(3 * (size_t)n);
    auto need_n = [&](long long m, const std::string& f) {
        if (m != n) throw ParseError(DSMC_ERR_PARSE, f + ": " + std::to_string(m) + " entries, positions has " +
                                                        std::to_string(n));
    };
    {
        ListTokens T;
        const std::string f = dir + "/U";
        if (!field_tokens(f, T)) throw ParseError(DSMC_ERR_IO, "cannot open " + f);
        P.U.assign(3 * (size_t)n, 0.0);
        need_n(read_list(T, f, [&](long long k) { double v[3]; read_vector(T, f, v);
                                                  if (k >= 0) for (int a = 0; a < 3; ++a) P.U[3 * k + a] = v[a]; }), f);
    }
    {
        ListTokens T;
        const std::string f = dir + "/typeId";
        if (!field_tokens(f, T)) throw ParseError(DSMC_ERR_IO, "cannot open " + f);
        P.species.assign((size_t)n, 0);
        need_n(read_list(T, f, [&](long long k) { const int v = (int)tok_num(T.take(), f); if (k >= 0) P.species[k] = v; }), f);
    }
    P.erot.assign((size_t)n, 0.0);
    {
        ListTokens T;
        const std::string f = dir + "/ERot";
        if (field_tokens(f, T))
            need_n(read_list(T, f, [&](long long k) { const double v = tok_num(T.take(), f); if (k >= 0) P.erot[k] = v; }), f);
    }
    P.vib.assign((size_t)n, 0);
    {
        ListTokens T;
        const std::string f = dir + "/vibLevel";
        if (field_tokens(f, T))
            need_n(read_list(T, f, [&](long long k) {
                       // a labelList per parcel: "m(l0 ...)" or "m{l}"; the first mode is kept
                       const long long m = (long long)tok_num(T.take(), f);
                       int first = 0;
                       if (T.peek().kind == Tok::PUNCT && T.peek().s == "{") {
                           T.take();
                           first = (int)tok_num(T.take(), f);
                           T.expect("}", f);
                       } else {
                           T.expect("(", f);
                           for (long long q = 0; q < m; ++q) {
                               const int v = (int)tok_num(T.take(), f);
                               if (q == 0) first = v;
                           }
                           T.expect(")", f);
                       }
                       if (m > 1) throw ParseError(DSMC_ERR_INVALID, f + ": more than one vibrational mode");
                       if (k >= 0) P.vib[k] = (m > 0) ? first : 0;
                   }), f);
    }
    P.id.resize((size_t)n);
    for (long long k = 0; k < n; ++k) P.id[k] = (unsigned)k;
    {
        ListTokens T;
        const std::string f = dir + "/origId";
        if (field_tokens(f, T))
            need_n(read_list(T, f, [&](long long k) { const long long v = (long long)tok_num(T.take(), f);
                                                      if (k >= 0) P.id[k] = (unsigned)v; }), f);
    }
}

}  // namespace

// internalField of a volScalarField: "uniform v" (one value) or
// "nonuniform List<scalar> N (...)".  False with err empty when the file
// does not exist.
bool dsmc::foam_read_scalar_field(const std::string& path, std::vector<double>& out, std::string& err) {
    err.clear();
    out.clear();
    try {
        ListTokens L;
        if (!field_tokens(path, L)) return false;
        while (L.peek().kind != Tok::END && !(L.peek().kind == Tok::WORD && L.peek().s == "internalField")) L.take();
        if (L.peek().kind == Tok::END) throw ParseError(DSMC_ERR_PARSE, path + ": no internalField");
        L.take();
        const Tok k = L.take();
        if (k.s == "uniform") {
            out.push_back(tok_num(L.take(), path));
            return true;
        }
        if (k.s != "nonuniform") throw ParseError(DSMC_ERR_PARSE, path + ": internalField is neither uniform nor nonuniform");
        L.take();   // List<scalar>
        out.resize(0);
        read_list(L, path, [&](long long i) {
            const double v = tok_num(L.take(), path);
            if (i >= 0) { if ((long long)out.size() <= i) out.resize((size_t)i + 1); out[(size_t)i] = v; }
        });
        return true;
    } catch (const std::exception& e) {
        err = e.what();
        return false;
    }
}

extern "C" int dsmc_parse_parcels(const char* case_dir, const char* time_name, const char* cloud_name, long long* n,
                                  double* pos, double* U, double* erot, int* vib, int* species, unsigned* id) {
    try {
        ParcelArrays P;
        read_parcel_files(std::string(case_dir) + "/" + time_name + "/lagrangian/" + cloud_name, P);
        const long long cap = *n;
        *n = P.n;
        if (!pos) return DSMC_OK;
        if (cap < P.n) throw ParseError(DSMC_ERR_CAPACITY, "arrays hold fewer entries than the cloud");
        std::memcpy(pos, P.pos.data(), sizeof(double) * P.pos.size());
        if (U) std::memcpy(U, P.U.data(), sizeof(double) * P.U.size());
        if (erot) std::memcpy(erot, P.erot.data(), sizeof(double) * P.erot.size());
        if (vib) std::memcpy(vib, P.vib.data(), sizeof(int) * P.vib.size());
        if (species) std::memcpy(species, P.species.data(), sizeof(int) * P.species.size());
        if (id) std::memcpy(id, P.id.data(), sizeof(unsigned) * P.id.size());
        return DSMC_OK;
    } catch (const ParseError& e) {
        g_perr = e.what();
        dsmc::set_global_error(g_perr);
        return e.code;
    } catch (const std::exception& e) {
        g_perr = e.what();
        dsmc::set_global_error(g_perr);
        return DSMC_ERR_PARSE;
    }
}

// ------------------------------------------------------------------ flux surfaces
// dsmcFluxSurface entries of system/fieldPropertiesDict (dsmcFluxSurface.C:
// 203-309: fieldName, faceZoneName, typeIds, fluxDirection) and the faceZone
// each names, from system/topoSetDict.
namespace {

const Node* topo_source(const Node* action) {
    const Node* si = action->find("sourceInfo");
    return si ? si : action;   // later OpenFOAM versions put the source keys in the action
}

// the box of faceSet `set`: exactly one action on it, "new" from boxToFace
void face_set_box(const Node& actions, const std::string& set, const std::string& where, double* lo, double* hi) {
    int found = 0;
    for (auto& a : actions.items) {
        if (a->kind != Node::DICT || wordOr(a.get(), "name", "") != set) continue;
        if (wordOr(a.get(), "type", "") != "faceSet") continue;
        ++found;
        const std::string act = wordOr(a.get(), "action", "");
        const std::string src = wordOr(a.get(), "source", "");
        if (act != "new" || src != "boxToFace")
            throw ParseError(DSMC_ERR_INVALID, "faceSet " + set + " in " + where +
                                                   ": only one 'action new; source boxToFace;' is supported");
        const Node& box = need(topo_source(a.get()), "box", "boxToFace of " + set);
        if (box.kind != Node::LIST || box.more.size() != 1)
            throw ParseError(DSMC_ERR_PARSE, "box of faceSet " + set + " is not '(min) (max)'");
        const auto a0 = numList(box, "box"), a1 = numList(*box.more[0], "box");
        if (a0.size() != 3 || a1.size() != 3) throw ParseError(DSMC_ERR_PARSE, "box of faceSet " + set + " is not two points");
        for (int k = 0; k < 3; ++k) {
            lo[k] = a0[k];
            hi[k] = a1[k];
        }
    }
    if (found != 1)
        throw ParseError(DSMC_ERR_INVALID, "Cannot find region: " + set + " in " + where +
                                               (found ? " (more than one action on the set)" : ""));
}

// faceZone `zone`: a faceZoneSet made by setToFaceZone from a faceSet, or a
// faceSet of that name (setsToZones makes a zone of every set)
void face_zone_box(const Node& actions, const std::string& zone, const std::string& where, double* lo, double* hi) {
    for (auto& a : actions.items) {
        if (a->kind != Node::DICT || wordOr(a.get(), "name", "") != zone) continue;
        if (wordOr(a.get(), "type", "") != "faceZoneSet") continue;
        if (wordOr(a.get(), "source", "") != "setToFaceZone")
            throw ParseError(DSMC_ERR_INVALID, "faceZoneSet " + zone + " in " + where +
                                                   ": only source setToFaceZone is supported");
        face_set_box(actions, word(topo_source(a.get()), "faceSet", "setToFaceZone of " + zone), where, lo, hi);
        return;
    }
    face_set_box(actions, zone, where, lo, hi);
}

void read_flux_surfaces(const std::string& dir, std::vector<dsmc_flux_surface>* out) {
    const std::string fpPath = dir + "/system/fieldPropertiesDict";
    {
        std::ifstream probe(fpPath);
        if (!probe) return;
    }
    auto fp = readDict(fpPath);
    const Node* fl = fp->find("dsmcFields");
    if (!fl) return;
    std::shared_ptr<Node> topo, dp;
    std::vector<std::string> types;
    for (auto& it : fl->items) {
        if (it->kind != Node::DICT || wordOr(it.get(), "fieldModel", "") != "dsmcFluxSurface") continue;
        if (!dp) {
            const std::string dpPath = fileIn(dir, "constant/dsmcProperties");
            dp = readDict(dpPath);
            types = wordList(need(dp.get(), "typeIdList", dpPath));
        }
        const Node& pr = need(it.get(), "dsmcFluxSurfaceProperties", fpPath);
        dsmc_flux_surface s;
        std::memset(&s, 0, sizeof(s));
        const std::string zone = word(&pr, "faceZoneName", "dsmcFluxSurfaceProperties");
        copyName(s.field_name, word(&pr, "fieldName", "dsmcFluxSurfaceProperties"));
        copyName(s.zone_name, zone);
        for (const std::string& t : wordList(need(&pr, "typeIds", "dsmcFluxSurfaceProperties"))) {
            const auto k = std::find(types.begin(), types.end(), t);
            if (k == types.end())
                throw ParseError(DSMC_ERR_INVALID, "Cannot find typeId: " + t + " in: " + fpPath);
            s.species_mask |= 1u << (unsigned)(k - types.begin());
        }
        const auto d = numList(need(&pr, "fluxDirection", "dsmcFluxSurfaceProperties"), "fluxDirection");
        if (d.size() != 3) throw ParseError(DSMC_ERR_PARSE, "fluxDirection is not a vector");
        for (int k = 0; k < 3; ++k) s.direction[k] = d[k];
        const std::string tsPath = dir + "/system/topoSetDict";
        if (!topo) topo = readDict(tsPath);
        face_zone_box(need(topo.get(), "actions", tsPath), zone, tsPath, s.box_min, s.box_max);
        out->push_back(s);
    }
}

}  // namespace

extern "C" int dsmc_parse_flux_surfaces(const char* case_dir, dsmc_flux_surface* out, int* n) {
    try {
        std::vector<dsmc_flux_surface> v;
        read_flux_surfaces(case_dir, &v);
        if (out) {
            if (*n < (int)v.size()) throw ParseError(DSMC_ERR_INVALID, "flux surface capacity too small");
            std::copy(v.begin(), v.end(), out);
        }
        *n = (int)v.size();
        return DSMC_OK;
    } catch (const ParseError& e) {
        g_perr = e.what();
        dsmc::set_global_error(g_perr);
        return e.code;
    } catch (const std::exception& e) {
        g_perr = e.what();
        dsmc::set_global_error(g_perr);
        return (g_perr.find("cannot open") != std::string::npos) ? DSMC_ERR_IO : DSMC_ERR_PARSE;
    }
}

extern "C" int dsmc_create(const char* case_dir, dsmc_handle** out) {
    *out = nullptr;
    dsmc_case_spec s;
    int rc = dsmc_parse_case(case_dir, &s);
    if (rc != DSMC_OK) return rc;
    int nS = 0;
    if ((rc = dsmc_parse_flux_surfaces(case_dir, nullptr, &nS)) != DSMC_OK) return rc;
    std::vector<dsmc_flux_surface> surf(nS);
    if (nS && (rc = dsmc_parse_flux_surfaces(case_dir, surf.data(), &nS)) != DSMC_OK) return rc;
    if ((rc = dsmc_create_from_spec(&s, out)) != DSMC_OK) return rc;
    for (const auto& f : surf) {
        if ((rc = dsmc_add_flux_surface(*out, &f)) != DSMC_OK) {
            dsmc::set_global_error(dsmc_last_error(*out));
            dsmc_destroy(*out);
            *out = nullptr;
            return rc;
        }
    }
    return DSMC_OK;
}
