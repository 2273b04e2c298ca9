"""Host-side rules of the MultiLevel merge strategies (the reference's
src/indices/multilevel/merge.jl:79-169 and the BoundedMaxHeap of
src/utils/neighbor_heaps.jl:84-190), including the known answer of the
merge_results docstring (merge.jl:63-72)."""


def test_merge_rules_on_ties_and_duplicates():
    # host-side rules: SimpleMerge keeps the first occurrence of an id after a
    # stable sort; DisjointMerge admits strictly closer points once full
    from manifoldann_gb300 import multilevel as ML
    from manifoldann_gb300.indices import Neighbor as N

    lists = [[N(10, 0.5), N(20, 0.8)], [N(30, 0.3), N(40, 1.2)], [N(50, 0.6)]]
    assert [n.id for n in ML.merge_results(ML.SimpleMerge(), lists, 3)] == [30, 10, 50]
    dup = [[N(7, 0.2), N(8, 0.5)], [N(7, 0.2), N(9, 0.5)]]
    assert [n.id for n in ML.merge_results(ML.SimpleMerge(), dup, 3)] == [7, 8, 9]
    ties = [[N(5, 1.0), N(3, 1.0)], [N(4, 1.0), N(1, 0.5)]]
    assert [n.id for n in ML.merge_results(ML.SimpleMerge(), ties, 3)] == [1, 5, 3]
    # heap: 5, 3 in; 4 (1.0) not < max 1.0 -> rejected; 1 replaces the max
    assert [n.id for n in ML.merge_results(ML.DisjointMerge(), ties, 2)] == [1, 3]
    assert ML.merge_results(ML.DisjointMerge(), [[], []], 4) == []
