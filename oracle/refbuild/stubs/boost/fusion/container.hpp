// Stand-in for the small part of Boost.Fusion the reference uses: a type
// list (vector), a keyed list of type lists (map of pairs), at_key and
// for_each over default-constructed elements (oracle build only).
#pragma once
#include <type_traits>
namespace boost { namespace fusion {
template <class... T> struct vector {};
template <class K, class V> struct pair { using key = K; using value = V; };
template <class... P> struct map {};
namespace detail {
template <class K, class... P> struct find_key;
template <class K, class V, class... R> struct find_key<K, pair<K, V>, R...> { using type = V; };
template <class K, class P0, class... R> struct find_key<K, P0, R...> : find_key<K, R...> {};
}
template <class K, class... P> typename detail::find_key<K, P...>::type at_key(const map<P...>&) {
    return typename detail::find_key<K, P...>::type{};
}
template <class... T, class F> void for_each(const vector<T...>&, const F& f) {
    int dummy[] = {0, (f(T{}), 0)...};
    (void)dummy;
}
} }
