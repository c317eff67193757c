// Input-deck model: the same blocks, keys and defaults as Quicksilver's
// Parameters (Parameters.hh:12-175), so that a reference deck drops in.
#pragma once

#include <cstdint>
#include <map>
#include <string>
#include <vector>

#include "qsg.h"

namespace qsg {

struct GeometrySpec {          // GeometryParameters, Parameters.hh:12-43
    enum Shape { UNDEFINED, BRICK, SPHERE };
    std::string material;
    Shape shape = UNDEFINED;
    double radius = 0.0, x_center = 0.0, y_center = 0.0, z_center = 0.0;
    double x_min = 0.0, y_min = 0.0, z_min = 0.0, x_max = 0.0, y_max = 0.0, z_max = 0.0;
};

struct MaterialSpec {          // MaterialParameters, Parameters.hh:45-74
    std::string name;
    double mass = 1000.0;
    double total_cross_section = 1.0;
    int n_isotopes = 10;
    int n_reactions = 9;
    double source_rate = 0.0;
    std::string scattering_cross_section, absorption_cross_section, fission_cross_section;
    double scattering_ratio = 1.0, absorption_ratio = 1.0, fission_ratio = 1.0;
};

struct CrossSectionSpec {      // CrossSectionParameters, Parameters.hh:76-95
    std::string name;
    double aa = 0.0, bb = 0.0, cc = 0.0, dd = 0.0, ee = 1.0;
    double nu_bar = 2.4;
};

struct SimulationSpec {        // SimulationParameters, Parameters.hh:97-167
    std::string input_file;        // the deck file read (qsg_deck_parse_file)
    std::string boundary_condition = "reflect";
    std::string energy_spectrum;   // output file stem of the census energy spectrum ("" = none)
    std::string cross_sections_out;  // kept and echoed; this library writes no cross-section file
    int cycle_timers = 0, debug_threads = 0;   // kept and echoed (no effect here)
    int load_balance = 0;
    uint64_t n_particles = 1000000;
    uint64_t batch_size = 0;
    uint64_t n_batches = 10;
    int n_steps = 10;
    int nx = 10, ny = 10, nz = 10;
    int seed = 1029384756;
    int x_dom = 0, y_dom = 0, z_dom = 0;
    double dt = 1e-8;
    double f_max = 0.1;
    double lx = 100.0, ly = 100.0, lz = 100.0;
    double e_min = 1e-9, e_max = 20;
    int n_groups = 230;
    double low_weight_cutoff = 0.001;
    int balance_replications = 1, flux_replications = 1, cell_replications = 1;
    int coral_benchmark = 0;
};

struct Deck {
    SimulationSpec sim;
    std::vector<GeometrySpec> geometry;
    std::map<std::string, MaterialSpec> materials;        // sorted by name, as std::map in Parameters.hh:173
    std::map<std::string, CrossSectionSpec> cross_sections;
    bool defaults_supplied = false;
};

// Parse deck text; throws std::runtime_error on malformed input.
void parse_deck_text(const std::string& text, Deck& deck);
// supplyDefaults, Parameters.cc:350-379.
void supply_defaults(Deck& deck);
// Apply one Simulation key (command-line override); throws on bad value.
void set_simulation_key(Deck& deck, const std::string& key, const std::string& value);
// printParameters, Parameters.cc:97-215: the deck as the reference echoes it.
std::string deck_text(const Deck& deck);
int boundary_condition_code(const std::string& bc);

}  // namespace qsg

struct QsgDeck {
    qsg::Deck deck;
};
