// force_calculator_barnes_hut.hpp -- Barnes-Hut calculator of the reference's
// API (CUDA/include/force_calculator_barnes_hut.hpp:5-128).  Backed by the
// engine's Morton-octree pipeline; leaf_capacity is honoured.  The data
// members keep the reference's layout; the tree buffers among them are left
// empty (the engine owns its tree).
#pragma once
#include "force_calculator.hpp"

struct Bounds {
    float xmin, xmax;
    float ymin, ymax;
    float zmin, zmax;
    float size;
};

struct TreeArrays {
    float *center_x, *center_y, *center_z;
    float *size, *size_sqr;
    float *mass;
    float *com_x, *com_y, *com_z;
    int *first_child;
    int *parent;
    int *particle_count;
    int *particle_start;
    int *node_depth;
};

struct BarnesHutForceCalculator : public ForceCalculator {
    double softening_squared;
    double theta_sqr;
    int leaf_capacity;

    cudaEvent_t startEvent, stopEvent;
    double total_compute_time_ms;
    double build_tree_time_ms;
    double destroy_tree_time_ms;
    double traverse_tree_time_ms;

    Bounds *d_bounding_cube = nullptr;
    void *bounding_box_temp_storage = nullptr;
    size_t bounding_box_temp_storage_bytes = 0;
    void *radix_sort_temp_storage = nullptr;
    size_t radix_sort_temp_storage_bytes = 0;

    TreeArrays tree{};
    int *nextFreeNode = nullptr;

    int *level_node_ids[constant::MAX_DEPTH] = {nullptr};
    int level_counts[constant::MAX_DEPTH] = {0};

public:
    BarnesHutForceCalculator(double softening, double theta,
                             int leaf_capacity = constant::LEAF_CAPACITY)
        : softening_squared(softening * softening), theta_sqr(theta * theta),
          leaf_capacity(leaf_capacity), startEvent(nullptr), stopEvent(nullptr),
          total_compute_time_ms(0.0), build_tree_time_ms(0.0), destroy_tree_time_ms(0.0),
          traverse_tree_time_ms(0.0)
    {
    }
    ~BarnesHutForceCalculator() = default;

    void computeAccelerations(ParticleArrays &particles) override;

    // The engine's build is one pipeline (bounding box, Morton codes, sort,
    // octree, monopoles); each of these runs the whole build of the current
    // positions.  destroyTree is a no-op (the tree is rebuilt per call).
    void buildTree(ParticleArrays &particles);
    void computeBoundingBox(ParticleArrays &particles);
    void radixSort(ParticleArrays &particles);
    void buildOctree(const uint32_t *sorted_morton_codes, int num_particles, TreeArrays &tree,
                     int *d_next_free_node);
    void computeMassCOM(ParticleArrays &particles);
    void destroyTree();

    std::string name() const override { return "Barnes-Hut"; }
    double getTotalComputeTime() const { return total_compute_time_ms; }
    double getBuildTreeTime() const { return build_tree_time_ms; }
    double getDestroyTreeTime() const { return destroy_tree_time_ms; }
    double getTraversalTime() const { return traverse_tree_time_ms; }
    void resetTimeStatistics()
    {
        total_compute_time_ms = 0.0;
        build_tree_time_ms = 0.0;
        destroy_tree_time_ms = 0.0;
        traverse_tree_time_ms = 0.0;
    }
};
