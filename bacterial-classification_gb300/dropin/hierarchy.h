// Taxonomy tree + FASTA store with the public interface of the reference's
// src/hierarchy.h:8-29 (class Hierarchy).  Host support for the GPU
// propagate-children driver.  The containers and the order of insertions
// follow the reference, so get_order() and get_children() iterate in the
// same order on the same standard library -- propagate-children's greedy
// selection depends on that order.
#pragma once
#include <filesystem>
#include <string>
#include <unordered_map>
#include <vector>

class Hierarchy {
public:
    Hierarchy(std::string seq_dir, std::string taxes);
    const std::vector<std::string>& get_sequences(std::string category);
    void append_sequence(std::string category, std::string seq);
    std::vector<std::string> get_order(std::string order);
    const std::vector<std::string>* get_children(std::string category);

private:
    std::string make_seq_id(const std::string& category);
    std::filesystem::path seq_dir;
    std::string taxes;
    std::unordered_map<std::string, std::vector<std::string>> children;
    std::unordered_map<std::string, std::vector<std::string>> seq_cache;
};
