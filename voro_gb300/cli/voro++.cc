// voro++: the reference's command-line utility (src/cmd_line.cc:166-497) on
// the GPU engine, through the drop-in header.
//
//   voro++ [options] <x_min> <x_max> <y_min> <y_max> <z_min> <z_max> <filename>
//
// reads "id x y z" (with -r: "id x y z r") per line from <filename>, computes
// every Voronoi cell and writes <filename.vol>, one print_custom line per
// cell ("%i %q %v", with -r "%i %q %v %r", or the -c string), in the
// reference's loop order or, with -o, in the order of the file.  Options,
// their defaults, error messages and exit codes are the reference's:
// -c -g -h -hc -l -m -n -o -p -px -py -pz -r -v --version -wb -wc -wo -ws -wp
// -y -yp -yv.  The grid of blocks only fixes the loop order here (the engine
// searches on its own grid); it is chosen as the reference chooses it:
// guess_optimal (src/pre_container.cc:57-63), -l or -n.  -g and -y/-yv draw
// every edge of every cell once (gnuplot segments, POV-Ray spheres and
// cylinders); the reference draws the same edges in the order of its own
// vertex tables.
#include <cfloat>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <type_traits>
#include <vector>

#include "../../include/voro_gb300.hh"

using namespace voro;

namespace {

constexpr int kMaxRegions = 16777216;             // the reference's cap on grid blocks
constexpr double kOptimalParticles = 5.6;         // particles per block, src/config.hh:97
constexpr double kTolerance = 10.0 * DBL_EPSILON;  // src/config.hh:80: the length-scale floor of -l

void help_message() {
    puts("Voro++ version 0.4.6 (GB300 engine)\n\n"
         "Syntax: voro++ [options] <x_min> <x_max> <y_min>\n"
         "               <y_max> <z_min> <z_max> <filename>\n\n"
         "By default, the utility reads in the input file of particle IDs and positions,\n"
         "computes the Voronoi cell for each, and then creates <filename.vol> with an\n"
         "additional column containing the volume of each Voronoi cell.\n\n"
         "Available options:\n"
         " -c <str>   : Specify a custom output string\n"
         " -g         : Turn on the gnuplot output to <filename.gnu>\n"
         " -h/--help  : Print this information\n"
         " -hc        : Print information about custom output\n"
         " -l <len>   : Manually specify a length scale to configure the internal\n"
         "              computational grid\n"
         " -m <mem>   : Manually choose the memory allocation per grid block\n"
         "              (default 8)\n"
         " -n [3]     : Manually specify the internal grid size\n"
         " -o         : Ensure that the output file has the same order as the input\n"
         "              file\n"
         " -p         : Make container periodic in all three directions\n"
         " -px        : Make container periodic in the x direction\n"
         " -py        : Make container periodic in the y direction\n"
         " -pz        : Make container periodic in the z direction\n"
         " -r         : Assume the input file has an extra coordinate for radii\n"
         " -v         : Verbose output\n"
         " --version  : Print version information\n"
         " -wb [6]    : Add six plane wall objects to make rectangular box containing\n"
         "              the space x1<x<x2, x3<y<x4, x5<z<x6\n"
         " -wc [7]    : Add a cylinder wall object, centered on (x1,x2,x3),\n"
         "              pointing in (x4,x5,x6), radius x7\n"
         " -wo [7]    : Add a conical wall object, apex at (x1,x2,x3), axis\n"
         "              along (x4,x5,x6), angle x7 in radians\n"
         " -ws [4]    : Add a sphere wall object, centered on (x1,x2,x3),\n"
         "              with radius x4\n"
         " -wp [4]    : Add a plane wall object, with normal (x1,x2,x3),\n"
         "              and displacement x4\n"
         " -y         : Save POV-Ray particles to <filename_p.pov> and POV-Ray Voronoi\n"
         "              cells to <filename_v.pov>\n"
         " -yp        : Save only POV-Ray particles to <filename_p.pov>\n"
         " -yv        : Save only POV-Ray Voronoi cells to <filename_v.pov>");
}

void custom_output_message() {
    puts("The \"-c\" option allows a string to be specified that will customize the output\n"
         "file to contain a variety of statistics about each computed Voronoi cell. The\n"
         "string is similar to the standard C printf() function, made up of text with\n"
         "additional control sequences that begin with percentage signs that are expanded\n"
         "to different statistics.\n"
         "\nParticle-related:\n"
         "  %i The particle ID number\n"
         "  %x The x coordinate of the particle\n"
         "  %y The y coordinate of the particle\n"
         "  %z The z coordinate of the particle\n"
         "  %q The position vector of the particle, short for \"%x %y %z\"\n"
         "  %r The radius of the particle (only printed if -p enabled)\n"
         "\nVertex-related:\n"
         "  %w The number of vertices in the Voronoi cell\n"
         "  %p A list of the vertices of the Voronoi cell in the format (x,y,z),\n"
         "     relative to the particle center\n"
         "  %P A list of the vertices of the Voronoi cell in the format (x,y,z),\n"
         "     relative to the global coordinate system\n"
         "  %o A list of the orders of each vertex\n"
         "  %m The maximum radius squared of a vertex position, relative to the\n"
         "     particle center\n"
         "\nEdge-related:\n"
         "  %g The number of edges of the Voronoi cell\n"
         "  %E The total edge distance\n"
         "  %e A list of perimeters of each face\n"
         "\nFace-related:\n"
         "  %s The number of faces of the Voronoi cell\n"
         "  %F The total surface area of the Voronoi cell\n"
         "  %A A frequency table of the number of edges for each face\n"
         "  %a A list of the number of edges for each face\n"
         "  %f A list of areas of each face\n"
         "  %t A list of bracketed sequences of vertices that make up each face\n"
         "  %l A list of normal vectors for each face\n"
         "  %n A list of neighboring particle or wall IDs corresponding to each face\n"
         "\nVolume-related:\n"
         "  %v The volume of the Voronoi cell\n"
         "  %c The centroid of the Voronoi cell, relative to the particle center\n"
         "  %C The centroid of the Voronoi cell, in the global coordinate system");
}

void version_message() { puts("Voro++ version 0.4.6 (GB300 engine)"); }

void error_message() {
    fputs("voro++: Unrecognized command-line options; type \"voro++ -h\" for more\ninformation.\n", stderr);
}

struct Options {
    int custom = 0;   // argv index of the -c string
    bool gnuplot = false, povp = false, povv = false, poly = false, ordered = false, verbose = false;
    bool per[3] = {false, false, false};
    enum { kNone, kLength, kSpecified } grid = kNone;
    double ls = 0;
    int n[3] = {0, 0, 0};
    int init_mem = 8;
    std::vector<std::pair<int, std::vector<double>>> walls;   // (VGPU_WALL_*, parameters); IDs -7, -8, ...
};

// The input's particles.  pre_container::put (src/pre_container.cc:71-80)
// keeps the ones inside the box along every non-periodic axis (ends
// included), and guess_optimal counts those; the container's own put() then
// drops what lies outside its blocks, as here.
struct Particle {
    int id;
    double x, y, z, r;
};

bool read_particles(const char *fn, bool with_r, std::vector<Particle> &out) {
    FILE *fp = fopen(fn, "r");
    if (!fp) {
        fprintf(stderr, "voro++: Unable to open file '%s'\n", fn);
        return false;
    }
    Particle p{0, 0, 0, 0, 0.5};
    int got;
    while ((got = with_r ? fscanf(fp, "%d %lg %lg %lg %lg", &p.id, &p.x, &p.y, &p.z, &p.r)
                         : fscanf(fp, "%d %lg %lg %lg", &p.id, &p.x, &p.y, &p.z)) == (with_r ? 5 : 4))
        out.push_back(p);
    fclose(fp);
    if (got != EOF) {
        fputs("voro++: File import error\n", stderr);
        return false;
    }
    return true;
}

template <class Con>
void add_walls(Con &con, const Options &o) {
    int j = -7;
    for (const auto &w : o.walls) {
        const std::vector<double> &a = w.second;
        switch (w.first) {
            case VGPU_WALL_PLANE: {
                wall_plane p(a[0], a[1], a[2], a[3], j);
                con.add_wall(p);
            } break;
            case VGPU_WALL_SPHERE: {
                wall_sphere p(a[0], a[1], a[2], a[3], j);
                con.add_wall(p);
            } break;
            case VGPU_WALL_CYLINDER: {
                wall_cylinder p(a[0], a[1], a[2], a[3], a[4], a[5], a[6], j);
                con.add_wall(p);
            } break;
            case VGPU_WALL_CONE: {
                wall_cone p(a[0], a[1], a[2], a[3], a[4], a[5], a[6], j);
                con.add_wall(p);
            } break;
        }
        j--;
    }
}

// every edge of the cell once (vertex index pairs a < b), from its face loops
void cell_edges(const voronoicell &c, std::vector<std::pair<int, int>> &edges) {
    std::vector<int> fv;
    c.face_vertices(fv);
    edges.clear();
    for (size_t i = 0; i < fv.size();) {
        const int m = fv[i++];
        for (int j = 0; j < m; j++) {
            const int a = fv[i + j], b = fv[i + (j + 1) % m];
            if (a < b) edges.emplace_back(a, b);   // each edge is on two faces, once in each direction
        }
        i += m;
    }
}

template <class Con, class Loop>
void run(Con &con, Loop &vl, const Options &o, const char *fmt, FILE *out, FILE *gnu, FILE *povp, FILE *povv,
         double &vol, int &vcc) {
    if (gnu || povv) con.set_polytopes(true);
    con.print_custom_loop(vl, fmt, out);
    if (!(gnu || povp || povv || o.verbose)) return;
    voronoicell_neighbor c;
    std::vector<double> v;
    std::vector<std::pair<int, int>> edges;
    if (vl.start()) do {
            if (!con.compute_cell(c, vl)) continue;
            int pid;
            double x, y, z, r;
            vl.pos(pid, x, y, z, r);
            if (gnu || povv) {
                c.vertices(x, y, z, v);
                cell_edges(c, edges);
            }
            if (gnu)
                for (const auto &e : edges)
                    fprintf(gnu, "%g %g %g\n%g %g %g\n\n\n", v[3 * e.first], v[3 * e.first + 1], v[3 * e.first + 2],
                            v[3 * e.second], v[3 * e.second + 1], v[3 * e.second + 2]);
            if (povp) {
                fprintf(povp, "// id %d\n", pid);
                if (o.poly) fprintf(povp, "sphere{<%g,%g,%g>,%g}\n", x, y, z, r);
                else fprintf(povp, "sphere{<%g,%g,%g>,s}\n", x, y, z);
            }
            if (povv) {
                fprintf(povv, "// cell %d\n", pid);
                for (size_t i = 0; i < v.size(); i += 3) fprintf(povv, "sphere{<%g,%g,%g>,r}\n", v[i], v[i + 1], v[i + 2]);
                for (const auto &e : edges)
                    fprintf(povv, "cylinder{<%g,%g,%g>,<%g,%g,%g>,r}\n", v[3 * e.first], v[3 * e.first + 1],
                            v[3 * e.first + 2], v[3 * e.second], v[3 * e.second + 1], v[3 * e.second + 2]);
            }
            if (o.verbose) {
                vol += c.volume();
                vcc++;
            }
        } while (vl.inc());
}

template <class Con>
void compute(Con &con, const Options &o, const std::vector<Particle> &pts, const char *fmt, FILE *out, FILE *gnu,
             FILE *povp, FILE *povv, double &vol, int &vcc, int &tp) {
    add_walls(con, o);
    particle_order vo;
    for (const Particle &p : pts) {
        if constexpr (std::is_same<Con, container_poly>::value) {
            if (o.ordered) con.put(vo, p.id, p.x, p.y, p.z, p.r);
            else con.put(p.id, p.x, p.y, p.z, p.r);
        } else {
            if (o.ordered) con.put(vo, p.id, p.x, p.y, p.z);
            else con.put(p.id, p.x, p.y, p.z);
        }
    }
    if (o.ordered) {
        c_loop_order vl(con, vo);
        run(con, vl, o, fmt, out, gnu, povp, povv, vol, vcc);
    } else {
        c_loop_all vl(con);
        run(con, vl, o, fmt, out, gnu, povp, povv, vol, vcc);
    }
    tp = con.total_particles();
}

}  // namespace

int main(int argc, char **argv) {
    Options o;
    if (argc == 2) {
        if (strcmp(argv[1], "-h") == 0 || strcmp(argv[1], "--help") == 0) {
            help_message();
            return 0;
        } else if (strcmp(argv[1], "-hc") == 0) {
            custom_output_message();
            return 0;
        } else if (strcmp(argv[1], "--version") == 0) {
            version_message();
            return 0;
        }
        error_message();
        return VOROPP_CMD_LINE_ERROR;
    }
    if (argc < 7) {
        error_message();
        return VOROPP_CMD_LINE_ERROR;
    }
    int i = 1;
    // an option with k values must leave them and the seven trailing arguments
    auto need = [&](int k) { return i < argc - 7 - k; };
    while (i < argc - 7) {
        const char *a = argv[i];
        if (strcmp(a, "-c") == 0) {
            if (!need(1)) {
                error_message();
                return VOROPP_CMD_LINE_ERROR;
            }
            if (o.custom != 0) {
                fputs("voro++: multiple custom output strings detected\n", stderr);
                return VOROPP_CMD_LINE_ERROR;
            }
            o.custom = ++i;
        } else if (strcmp(a, "-g") == 0) {
            o.gnuplot = true;
        } else if (strcmp(a, "-h") == 0 || strcmp(a, "--help") == 0) {
            help_message();
            return 0;
        } else if (strcmp(a, "-hc") == 0) {
            custom_output_message();
            return 0;
        } else if (strcmp(a, "-l") == 0) {
            if (!need(1)) {
                error_message();
                return VOROPP_CMD_LINE_ERROR;
            }
            if (o.grid != Options::kNone) {
                fputs("voro++: Conflicting options about grid setup (-l/-n)\n", stderr);
                return VOROPP_CMD_LINE_ERROR;
            }
            o.grid = Options::kLength;
            o.ls = atof(argv[++i]);
        } else if (strcmp(a, "-m") == 0) {
            o.init_mem = atoi(argv[++i]);
        } else if (strcmp(a, "-n") == 0) {
            if (!need(3)) {
                error_message();
                return VOROPP_CMD_LINE_ERROR;
            }
            if (o.grid != Options::kNone) {
                fputs("voro++: Conflicting options about grid setup (-l/-n)\n", stderr);
                return VOROPP_CMD_LINE_ERROR;
            }
            o.grid = Options::kSpecified;
            for (int a3 = 0; a3 < 3; a3++) o.n[a3] = atoi(argv[++i]);
            if (o.n[0] <= 0 || o.n[1] <= 0 || o.n[2] <= 0) {
                fputs("voro++: Computational grid specified with -n must be greater than one\n"
                      "in each direction\n",
                      stderr);
                return VOROPP_CMD_LINE_ERROR;
            }
        } else if (strcmp(a, "-o") == 0) {
            o.ordered = true;
        } else if (strcmp(a, "-p") == 0) {
            o.per[0] = o.per[1] = o.per[2] = true;
        } else if (strcmp(a, "-px") == 0) {
            o.per[0] = true;
        } else if (strcmp(a, "-py") == 0) {
            o.per[1] = true;
        } else if (strcmp(a, "-pz") == 0) {
            o.per[2] = true;
        } else if (strcmp(a, "-r") == 0) {
            o.poly = true;
        } else if (strcmp(a, "-v") == 0) {
            o.verbose = true;
        } else if (strcmp(a, "--version") == 0) {
            version_message();
            return 0;
        } else if (strcmp(a, "-wb") == 0 || strcmp(a, "-ws") == 0 || strcmp(a, "-wp") == 0 ||
                   strcmp(a, "-wc") == 0 || strcmp(a, "-wo") == 0) {
            const int k = a[2] == 'b' ? 6 : (a[2] == 's' || a[2] == 'p' ? 4 : 7);
            if (!need(k)) {
                error_message();
                return VOROPP_CMD_LINE_ERROR;
            }
            std::vector<double> w(k);
            for (int q = 0; q < k; q++) w[q] = atof(argv[++i]);
            if (a[2] == 'b') {   // six planes bounding x1<x<x2, x3<y<x4, x5<z<x6
                o.walls.push_back({VGPU_WALL_PLANE, {-1, 0, 0, -w[0]}});
                o.walls.push_back({VGPU_WALL_PLANE, {1, 0, 0, w[1]}});
                o.walls.push_back({VGPU_WALL_PLANE, {0, -1, 0, -w[2]}});
                o.walls.push_back({VGPU_WALL_PLANE, {0, 1, 0, w[3]}});
                o.walls.push_back({VGPU_WALL_PLANE, {0, 0, -1, -w[4]}});
                o.walls.push_back({VGPU_WALL_PLANE, {0, 0, 1, w[5]}});
            } else {
                const int t = a[2] == 's'   ? VGPU_WALL_SPHERE
                              : a[2] == 'p' ? VGPU_WALL_PLANE
                              : a[2] == 'c' ? VGPU_WALL_CYLINDER
                                            : VGPU_WALL_CONE;
                o.walls.push_back({t, w});
            }
        } else if (strcmp(a, "-y") == 0) {
            o.povp = o.povv = true;
        } else if (strcmp(a, "-yp") == 0) {
            o.povp = true;
        } else if (strcmp(a, "-yv") == 0) {
            o.povv = true;
        } else {
            error_message();
            return VOROPP_CMD_LINE_ERROR;
        }
        i++;
    }
    if (o.init_mem <= 0) {
        fputs("voro++: The memory allocation must be positive\n", stderr);
        return VOROPP_CMD_LINE_ERROR;
    }
    const double ax = atof(argv[i]), bx = atof(argv[i + 1]), ay = atof(argv[i + 2]), by = atof(argv[i + 3]),
                 az = atof(argv[i + 4]), bz = atof(argv[i + 5]);
    const char *axes = "xyz";
    const double lo[3] = {ax, ay, az}, hi[3] = {bx, by, bz};
    for (int a = 0; a < 3; a++)
        if (hi[a] < lo[a]) {
            fprintf(stderr, "voro++: Minimum %c coordinate exceeds maximum %c coordinate\n", axes[a], axes[a]);
            return VOROPP_CMD_LINE_ERROR;
        }
    const char *fn = argv[i + 6];
    std::vector<Particle> pts;
    int nx, ny, nz;
    if (o.grid == Options::kNone) {
        // the file is read first, as the reference's pre_container imports it
        if (!read_particles(fn, o.poly, pts)) return VOROPP_FILE_ERROR;
        int64_t kept = 0;
        for (const Particle &p : pts) {
            const double c[3] = {p.x, p.y, p.z};
            bool in = true;
            for (int a = 0; a < 3; a++)
                if (!o.per[a] && !(c[a] >= lo[a] && c[a] <= hi[a])) in = false;
            kept += in;
        }
        const double dx = bx - ax, dy = by - ay, dz = bz - az;
        const double il = std::pow((double)kept / (kOptimalParticles * dx * dy * dz), 1 / 3.0);
        nx = int(dx * il + 1);
        ny = int(dy * il + 1);
        nz = int(dz * il + 1);
    } else {
        double nxf, nyf, nzf;
        if (o.grid == Options::kLength) {
            if (o.ls < kTolerance) {
                fputs("voro++: ", stderr);
                if (o.ls < 0) fputs("The length scale must be positive\n", stderr);
                else
                    fprintf(stderr,
                            "The length scale is smaller than the safe limit of %g. Either\nincrease the particle "
                            "length scale, or recompile with a different limit.\n",
                            kTolerance);
                return VOROPP_CMD_LINE_ERROR;
            }
            const double ls = 0.6 / o.ls;
            nxf = (bx - ax) * ls + 1;
            nyf = (by - ay) * ls + 1;
            nzf = (bz - az) * ls + 1;
            nx = int(nxf);
            ny = int(nyf);
            nz = int(nzf);
        } else {
            nx = o.n[0];
            ny = o.n[1];
            nz = o.n[2];
            nxf = nx;
            nyf = ny;
            nzf = nz;
        }
        if (nxf * nyf * nzf > kMaxRegions) {
            fprintf(stderr,
                    "voro++: Number of computational blocks exceeds the maximum allowed of %d.\n"
                    "Either increase the particle length scale, or recompile with an increased\nmaximum.",
                    kMaxRegions);
            return VOROPP_MEMORY_ERROR;
        }
    }
    if (strlen(fn) > 4096) {
        fputs("voro++: Filename too long\n", stderr);
        return VOROPP_CMD_LINE_ERROR;
    }
    if (o.grid != Options::kNone && !read_particles(fn, o.poly, pts)) return VOROPP_FILE_ERROR;
    auto open = [&](const char *suffix) -> FILE * {
        const std::string name = std::string(fn) + suffix;
        FILE *f = fopen(name.c_str(), "w");
        if (!f) {
            fprintf(stderr, "voro++: Unable to open file '%s'\n", name.c_str());
            exit(VOROPP_FILE_ERROR);
        }
        return f;
    };
    FILE *out = open(".vol");
    FILE *gnu = o.gnuplot ? open(".gnu") : nullptr;
    FILE *povp = o.povp ? open("_p.pov") : nullptr;
    FILE *povv = o.povv ? open("_v.pov") : nullptr;
    const char *fmt = o.custom == 0 ? (o.poly ? "%i %q %v %r" : "%i %q %v") : argv[o.custom];
    double vol = 0;
    int tp = 0, vcc = 0;
    if (o.poly) {
        container_poly con(ax, bx, ay, by, az, bz, nx, ny, nz, o.per[0], o.per[1], o.per[2], o.init_mem);
        compute(con, o, pts, fmt, out, gnu, povp, povv, vol, vcc, tp);
    } else {
        container con(ax, bx, ay, by, az, bz, nx, ny, nz, o.per[0], o.per[1], o.per[2], o.init_mem);
        compute(con, o, pts, fmt, out, gnu, povp, povv, vol, vcc, tp);
    }
    if (o.verbose) {
        printf("Container geometry        : [%g:%g] [%g:%g] [%g:%g]\n"
               "Computational grid size   : %d by %d by %d (%s)\n"
               "Filename                  : %s\n"
               "Output string             : %s%s\n",
               ax, bx, ay, by, az, bz, nx, ny, nz,
               o.grid == Options::kNone     ? "estimated from file"
               : o.grid == Options::kLength ? "estimated using length scale"
                                            : "directly specified",
               fn, fmt, o.custom == 0 ? " (default)" : "");
        printf("Total imported particles  : %d (%.2g per grid block)\n"
               "Total V. cells computed   : %d\n"
               "Total container volume    : %g\n"
               "Total V. cell volume      : %g\n",
               tp, ((double)tp) / (nx * ny * nz), vcc, (bx - ax) * (by - ay) * (bz - az), vol);
    }
    fclose(out);
    if (gnu) fclose(gnu);
    if (povp) fclose(povp);
    if (povv) fclose(povv);
    return 0;
}
