// Quicksilver input-deck reader.
//
// Line grammar (parseUtils.cc:17-87): a line is `keyword: value` or
// `keyword = value`; its indent is the count of leading white space.  A line
// with indent 0 and an empty value starts a block; the block's pairs are the
// following indented lines; comment lines (only white space and `//...`) are
// skipped inside a block.  Blocks are applied in file order
// (Parameters.cc:280-341) and a repeated key keeps its last value.  Values
// are read with operator>> like InputBlock::getValue (InputBlock.hh:35-47).
#include "deck.h"

#include <cctype>
#include <cstring>
#include <fstream>
#include <sstream>
#include <stdexcept>
#include <type_traits>

#include "status.h"

namespace qsg {

namespace {

const char* kWhitespace = " \t\f\v\n\r";

void chop(std::string& s)
{
    size_t here = s.size();
    while (here > 0 && isspace((unsigned char)s[here - 1])) --here;
    if (here < s.size()) s.erase(here);
    size_t n = 0;
    while (n < s.size() && isspace((unsigned char)s[n])) ++n;
    s.erase(0, n);
}

bool is_comment(std::string line)
{
    size_t here = line.find("//");
    if (here != std::string::npos) line.erase(here);
    return line.find_last_not_of(kWhitespace) == std::string::npos;
}

bool split(const std::string& line, std::string& keyword, std::string& value, int& indent)
{
    indent = 0;
    while (indent < (int)line.size() && isspace((unsigned char)line[indent])) ++indent;
    size_t delim = line.find_first_of(":=", indent);
    if (delim == std::string::npos) return false;
    keyword = line.substr(indent, delim - indent);
    chop(keyword);
    value.clear();
    if (delim + 1 < line.size()) {
        value = line.substr(delim + 1);
        chop(value);
    }
    return true;
}

struct Block {
    std::string name;
    std::map<std::string, std::string> kv;

    template <typename T>
    void get(const std::string& key, T& out) const
    {
        auto it = kv.find(key);
        if (it == kv.end()) return;
        if constexpr (std::is_same<T, std::string>::value) {
            // an empty string value: the reference's extraction fails and
            // qs_assert (which only prints) leaves the value "" -- the same
            // end result, taken here without the message, so that the
            // start-up echo (which prints empty strings) reads back
            if (it->second.find_first_not_of(" \t\r") == std::string::npos) {
                out.clear();
                return;
            }
        }
        std::istringstream in(it->second);
        T v{};
        in >> v;
        if (!in) throw std::runtime_error("deck: cannot parse " + name + "." + key + " = '" + it->second + "'");
        out = v;
    }
};

// readBlock, parseUtils.cc:31-49: returns the line that ended the block.
std::string read_block(Block& b, std::istream& in)
{
    std::string line;
    while (!in.eof()) {
        std::getline(in, line);
        if (is_comment(line)) continue;
        std::string k, v;
        int ind;
        if (!split(line, k, v, ind) || ind == 0) break;
        b.kv[k] = v;
    }
    return line;
}

// parseInputFile's scan loop, Parameters.cc:286-302.
std::vector<Block> parse_blocks(const std::string& text)
{
    std::vector<Block> blocks;
    std::istringstream in(text);
    std::string line;
    std::getline(in, line);
    while (!in.eof()) {
        std::string key, value;
        int indent;
        if (split(line, key, value, indent) && indent == 0 && value.empty()) {
            Block b;
            b.name = key;
            line = read_block(b, in);
            blocks.push_back(b);
        } else {
            std::getline(in, line);
        }
    }
    return blocks;
}

void scan_simulation(const Block& b, SimulationSpec& s)
{
    // Parameters.cc:384-418
    b.get("boundaryCondition", s.boundary_condition);
    b.get("dt", s.dt);
    b.get("fMax", s.f_max);
    b.get("loadBalance", s.load_balance);
    b.get("lx", s.lx);
    b.get("ly", s.ly);
    b.get("lz", s.lz);
    b.get("nParticles", s.n_particles);
    b.get("batchSize", s.batch_size);
    b.get("nBatches", s.n_batches);
    b.get("nSteps", s.n_steps);
    b.get("nx", s.nx);
    b.get("ny", s.ny);
    b.get("nz", s.nz);
    b.get("seed", s.seed);
    b.get("xDom", s.x_dom);
    b.get("yDom", s.y_dom);
    b.get("zDom", s.z_dom);
    b.get("eMax", s.e_max);
    b.get("eMin", s.e_min);
    b.get("nGroups", s.n_groups);
    b.get("lowWeightCutoff", s.low_weight_cutoff);
    b.get("bTally", s.balance_replications);
    b.get("fTally", s.flux_replications);
    b.get("cTally", s.cell_replications);
    b.get("coralBenchmark", s.coral_benchmark);
    b.get("energySpectrum", s.energy_spectrum);
    b.get("crossSectionsOut", s.cross_sections_out);
    b.get("cycleTimers", s.cycle_timers);
    b.get("debugThreads", s.debug_threads);
}

void scan_geometry(const Block& b, Deck& d)
{
    // Parameters.cc:423-450
    GeometrySpec g;
    b.get("material", g.material);
    std::string shape;
    b.get("shape", shape);
    if (shape == "brick") {
        g.shape = GeometrySpec::BRICK;
        b.get("xMax", g.x_max);
        b.get("xMin", g.x_min);
        b.get("yMax", g.y_max);
        b.get("yMin", g.y_min);
        b.get("zMax", g.z_max);
        b.get("zMin", g.z_min);
    } else if (shape == "sphere") {
        g.shape = GeometrySpec::SPHERE;
        b.get("radius", g.radius);
        b.get("xCenter", g.x_center);
        b.get("yCenter", g.y_center);
        b.get("zCenter", g.z_center);
    } else {
        throw std::runtime_error("deck: Geometry block needs shape brick or sphere");
    }
    d.geometry.push_back(g);
}

void scan_material(const Block& b, Deck& d)
{
    // Parameters.cc:454-473
    std::string name;
    b.get("name", name);
    if (name.empty()) throw std::runtime_error("deck: Material block without name");
    MaterialSpec& m = d.materials[name];
    m.name = name;
    b.get("mass", m.mass);
    b.get("absorptionCrossSection", m.absorption_cross_section);
    b.get("absorptionCrossSectionRatio", m.absorption_ratio);
    b.get("fissionCrossSection", m.fission_cross_section);
    b.get("fissionCrossSectionRatio", m.fission_ratio);
    b.get("nIsotopes", m.n_isotopes);
    b.get("nReactions", m.n_reactions);
    b.get("totalCrossSection", m.total_cross_section);
    b.get("scatteringCrossSection", m.scattering_cross_section);
    b.get("scatteringCrossSectionRatio", m.scattering_ratio);
    b.get("sourceRate", m.source_rate);
}

void scan_cross_section(const Block& b, Deck& d)
{
    // Parameters.cc:477-492
    std::string name;
    b.get("name", name);
    if (name.empty()) throw std::runtime_error("deck: CrossSection block without name");
    CrossSectionSpec& c = d.cross_sections[name];
    c.name = name;
    b.get("A", c.aa);
    b.get("B", c.bb);
    b.get("C", c.cc);
    b.get("D", c.dd);
    b.get("E", c.ee);
    b.get("nuBar", c.nu_bar);
}

}  // namespace

void parse_deck_text(const std::string& text, Deck& deck)
{
    for (const Block& b : parse_blocks(text)) {
        if (b.name == "Simulation") scan_simulation(b, deck.sim);
        if (b.name == "Geometry") scan_geometry(b, deck);
        if (b.name == "Material") scan_material(b, deck);
        if (b.name == "CrossSection") scan_cross_section(b, deck);
    }
}

void supply_defaults(Deck& deck)
{
    if (!deck.geometry.empty()) return;
    CrossSectionSpec flat;
    flat.name = "flat";
    deck.cross_sections[flat.name] = flat;
    MaterialSpec src;
    src.name = "sourceMaterial";
    src.mass = 1000.0;
    src.source_rate = 1e10;
    src.scattering_cross_section = "flat";
    src.absorption_cross_section = "flat";
    src.fission_cross_section = "flat";
    src.fission_ratio = 0.1;
    deck.materials[src.name] = src;
    GeometrySpec g;
    g.material = "sourceMaterial";
    g.shape = GeometrySpec::BRICK;
    g.x_max = deck.sim.lx;
    g.y_max = deck.sim.ly;
    g.z_max = deck.sim.lz;
    deck.geometry.push_back(g);
    deck.defaults_supplied = true;
}

void set_simulation_key(Deck& deck, const std::string& key, const std::string& value)
{
    Block b;
    b.name = "Simulation";
    b.kv[key] = value;
    static const char* known[] = {"boundaryCondition", "dt", "fMax", "loadBalance", "lx", "ly", "lz",
                                  "nParticles", "batchSize", "nBatches", "nSteps", "nx", "ny", "nz",
                                  "seed", "xDom", "yDom", "zDom", "eMax", "eMin", "nGroups",
                                  "lowWeightCutoff", "bTally", "fTally", "cTally", "coralBenchmark",
                                  "energySpectrum", "crossSectionsOut", "cycleTimers", "debugThreads"};
    bool ok = false;
    for (const char* k : known) ok = ok || key == k;
    if (!ok) throw std::runtime_error("deck: unknown Simulation key '" + key + "'");
    scan_simulation(b, deck.sim);
}

// The operator<< overloads of Parameters.cc:121-215, block by block, with the
// stream's default formatting, in the order printParameters writes them
// (geometries in deck order, materials and cross sections sorted by name).
// As there, a sphere's radius is not printed.
std::string deck_text(const Deck& d)
{
    std::ostringstream out;
    const SimulationSpec& s = d.sim;
    out << "Simulation:\n";
    out << "   dt: " << s.dt << "\n";
    out << "   fMax: " << s.f_max << "\n";
    out << "   inputFile: " << s.input_file << "\n";
    out << "   energySpectrum: " << s.energy_spectrum << "\n";
    out << "   boundaryCondition: " << s.boundary_condition << "\n";
    out << "   loadBalance: " << s.load_balance << "\n";
    out << "   cycleTimers: " << s.cycle_timers << "\n";
    out << "   debugThreads: " << s.debug_threads << "\n";
    out << "   lx: " << s.lx << "\n";
    out << "   ly: " << s.ly << "\n";
    out << "   lz: " << s.lz << "\n";
    out << "   nParticles: " << s.n_particles << "\n";
    out << "   batchSize: " << s.batch_size << "\n";
    out << "   nBatches: " << s.n_batches << "\n";
    out << "   nSteps: " << s.n_steps << "\n";
    out << "   nx: " << s.nx << "\n";
    out << "   ny: " << s.ny << "\n";
    out << "   nz: " << s.nz << "\n";
    out << "   seed: " << s.seed << "\n";
    out << "   xDom: " << s.x_dom << "\n";
    out << "   yDom: " << s.y_dom << "\n";
    out << "   zDom: " << s.z_dom << "\n";
    out << "   eMax: " << s.e_max << "\n";
    out << "   eMin: " << s.e_min << "\n";
    out << "   nGroups: " << s.n_groups << "\n";
    out << "   lowWeightCutoff: " << s.low_weight_cutoff << "\n";
    out << "   bTally: " << s.balance_replications << "\n";
    out << "   fTally: " << s.flux_replications << "\n";
    out << "   cTally: " << s.cell_replications << "\n";
    out << "   coralBenchmark: " << s.coral_benchmark << "\n";
    out << "   crossSectionsOut:" << s.cross_sections_out << "\n";
    out << "\n";
    for (const GeometrySpec& g : d.geometry) {
        out << "Geometry:\n";
        out << "   material: " << g.material << "\n";
        if (g.shape == GeometrySpec::BRICK) {
            out << "   shape: brick\n";
            out << "   xMax: " << g.x_max << "\n";
            out << "   xMin: " << g.x_min << "\n";
            out << "   yMax: " << g.y_max << "\n";
            out << "   yMin: " << g.y_min << "\n";
            out << "   zMax: " << g.z_max << "\n";
            out << "   zMin: " << g.z_min << "\n";
        } else {
            out << "   shape: sphere\n";
            out << "   xCenter: " << g.x_center << "\n";
            out << "   yCenter: " << g.y_center << "\n";
            out << "   zCenter: " << g.z_center << "\n";
        }
        out << "\n";
    }
    for (const auto& kv : d.materials) {
        const MaterialSpec& m = kv.second;
        out << "Material:\n";
        out << "   name: " << m.name << "\n";
        out << "   mass: " << m.mass << "\n";
        out << "   nIsotopes: " << m.n_isotopes << "\n";
        out << "   nReactions: " << m.n_reactions << "\n";
        out << "   sourceRate: " << m.source_rate << "\n";
        out << "   totalCrossSection: " << m.total_cross_section << "\n";
        out << "   absorptionCrossSection: " << m.absorption_cross_section << "\n";
        out << "   fissionCrossSection: " << m.fission_cross_section << "\n";
        out << "   scatteringCrossSection: " << m.scattering_cross_section << "\n";
        out << "   absorptionCrossSectionRatio: " << m.absorption_ratio << "\n";
        out << "   fissionCrossSectionRatio: " << m.fission_ratio << "\n";
        out << "   scatteringCrossSectionRatio: " << m.scattering_ratio << "\n";
        out << "\n";
    }
    for (const auto& kv : d.cross_sections) {
        const CrossSectionSpec& x = kv.second;
        out << "CrossSection:\n";
        out << "   name: " << x.name << "\n";
        out << "   A: " << x.aa << "\n";
        out << "   B: " << x.bb << "\n";
        out << "   C: " << x.cc << "\n";
        out << "   D: " << x.dd << "\n";
        out << "   E: " << x.ee << "\n";
        out << "   nuBar: " << x.nu_bar << "\n";
    }
    return out.str();
}

int boundary_condition_code(const std::string& bc)
{
    if (bc == "reflect") return 0;
    if (bc == "escape") return 1;
    if (bc == "octant") return 2;
    return -1;
}

}  // namespace qsg

extern "C" int qsg_deck_parse_string(const char* text, QsgDeck** out)
{
    QSG_API_BEGIN
    if (!text || !out) return qsg::fail(QSG_ERR_INVALID, "qsg_deck_parse_string: null argument");
    *out = nullptr;
    QsgDeck* d = new QsgDeck();
    try {
        qsg::parse_deck_text(text, d->deck);
        qsg::supply_defaults(d->deck);
    } catch (...) {
        delete d;
        throw;
    }
    *out = d;
    return QSG_OK;
    QSG_API_END
}

extern "C" int qsg_deck_parse_file(const char* path, QsgDeck** out)
{
    QSG_API_BEGIN
    if (!path || !out) return qsg::fail(QSG_ERR_INVALID, "qsg_deck_parse_file: null argument");
    std::ifstream in(path, std::ios::binary);
    if (!in) return qsg::fail(QSG_ERR_IO, "cannot open deck '%s'", path);
    std::stringstream ss;
    ss << in.rdbuf();
    std::string text = ss.str();
    const int st = qsg_deck_parse_string(text.c_str(), out);
    if (st == QSG_OK) (*out)->deck.sim.input_file = path;
    return st;
    QSG_API_END
}

extern "C" int qsg_deck_write(const QsgDeck* deck, char* buf, size_t len, size_t* needed)
{
    QSG_API_BEGIN
    if (!deck) return qsg::fail(QSG_ERR_INVALID, "qsg_deck_write: null deck");
    const std::string text = qsg::deck_text(deck->deck);
    if (needed) *needed = text.size() + 1;
    if (!buf || len < text.size() + 1)
        return qsg::fail(QSG_ERR_CAPACITY, "qsg_deck_write: the deck text needs %zu bytes", text.size() + 1);
    memcpy(buf, text.c_str(), text.size() + 1);
    return QSG_OK;
    QSG_API_END
}

extern "C" int qsg_deck_set(QsgDeck* deck, const char* key, const char* value)
{
    QSG_API_BEGIN
    if (!deck || !key || !value) return qsg::fail(QSG_ERR_INVALID, "qsg_deck_set: null argument");
    qsg::set_simulation_key(deck->deck, key, value);
    if (deck->deck.defaults_supplied) {
        // the default brick follows the box size (Parameters.cc:374-376)
        qsg::GeometrySpec& g = deck->deck.geometry[0];
        g.x_max = deck->deck.sim.lx;
        g.y_max = deck->deck.sim.ly;
        g.z_max = deck->deck.sim.lz;
    }
    return QSG_OK;
    QSG_API_END
}

extern "C" int qsg_deck_free(QsgDeck* deck)
{
    delete deck;
    return QSG_OK;
}

extern "C" int qsg_deck_energy_spectrum(const QsgDeck* deck, char* buf, size_t len)
{
    QSG_API_BEGIN
    if (!deck || !buf || len == 0) return qsg::fail(QSG_ERR_INVALID, "qsg_deck_energy_spectrum: null argument");
    const std::string& name = deck->deck.sim.energy_spectrum;
    if (name.size() + 1 > len) return qsg::fail(QSG_ERR_CAPACITY, "qsg_deck_energy_spectrum: buffer too small");
    std::memcpy(buf, name.c_str(), name.size() + 1);
    return QSG_OK;
    QSG_API_END
}

extern "C" int qsg_deck_simulation(const QsgDeck* deck, QsgSimulation* out)
{
    QSG_API_BEGIN
    if (!deck || !out) return qsg::fail(QSG_ERR_INVALID, "qsg_deck_simulation: null argument");
    const qsg::SimulationSpec& s = deck->deck.sim;
    *out = QsgSimulation{};
    out->dt = s.dt;
    out->lx = s.lx;
    out->ly = s.ly;
    out->lz = s.lz;
    out->e_min = s.e_min;
    out->e_max = s.e_max;
    out->low_weight_cutoff = s.low_weight_cutoff;
    out->n_particles = s.n_particles;
    out->batch_size = s.batch_size;
    out->n_batches = s.n_batches;
    out->n_steps = s.n_steps;
    out->nx = s.nx;
    out->ny = s.ny;
    out->nz = s.nz;
    out->seed = s.seed;
    out->x_dom = s.x_dom;
    out->y_dom = s.y_dom;
    out->z_dom = s.z_dom;
    out->n_groups = s.n_groups;
    out->load_balance = s.load_balance;
    out->balance_replications = s.balance_replications;
    out->flux_replications = s.flux_replications;
    out->cell_replications = s.cell_replications;
    out->coral_benchmark = s.coral_benchmark;
    out->boundary_condition = qsg::boundary_condition_code(s.boundary_condition);
    return QSG_OK;
    QSG_API_END
}
